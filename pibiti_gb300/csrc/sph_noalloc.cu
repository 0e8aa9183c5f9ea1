// sph_noalloc.cu -- RadixSort that allocates no device memory.
//
// Who needs it: callers that must not call cudaMalloc or cudaFree while they
// run.  cudaFree waits for the whole device to go idle and cudaMalloc can
// block on the driver, which a frame loop with a fixed time budget cannot
// afford; and a host process whose device memory is already held by another
// allocator (a framework's caching allocator, for example) may find no free
// memory for a fresh cudaMalloc at all.  sph_RadixSort grows a scratch buffer
// with cudaMalloc on first use and whenever a larger sort arrives; this
// variant never does.
//
// Its scratch is the file-scope array below: kNoAllocWords 32-bit words
// (2.0 MiB), which every GPU that loads this library holds until the process
// exits.  That covers sorts of up to kNoAllocMaxElements (4,194,304) pairs;
// larger requests are refused with SPH_ERR_ARG.  The device address of the
// array is looked up with cudaGetSymbolAddress (with the device current) on
// every call made outside a stream capture, and kept per device for calls
// made inside one: make one call on each device before capturing any stream.
// Looking it up again outside captures keeps the address right after a
// cudaDeviceReset, which reloads the module.  All calls share the one array
// and it keeps whatever the last
// call left there: the sort writes every histogram and offset entry before it
// reads them, and the scan's one counter word is cleared on the stream before
// each use.  Calls whose work overlaps on the GPU (two host threads, or two
// streams) race on the array; serialise them.
#include <mutex>

#include "sph_internal.h"

namespace sph {
namespace {

constexpr uint32_t kNoAllocMaxElements = 1u << 22;
// radix_scratch_words(kNoAllocMaxElements): two digit-major histograms of
// 256 x 1024 tiles plus the scan's counter and 64 tile sums (+3 spare).
constexpr size_t kNoAllocTiles = kNoAllocMaxElements / kScanTile;
constexpr size_t kNoAllocHist = 256 * kNoAllocTiles;
constexpr size_t kNoAllocWords = 2 * kNoAllocHist + 1 + (kNoAllocHist + kScanTile - 1) / kScanTile + 3;

static __device__ __align__(256) uint32_t g_radix_scratch[kNoAllocWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint32_t* g_scratch_addr[kMaxDevices] = {};

// Device address of g_radix_scratch on the current device: looked up when
// `stream` is not capturing (and kept), the kept one while it is.
int scratch_address(cudaStream_t stream, uint32_t** out) {
  int dev = 0;
  SPH_CUDA(cudaGetDevice(&dev), "RadixSort_noalloc: current device");
  if (dev < 0 || dev >= kMaxDevices) return fail(SPH_ERR_ARG, "RadixSort_noalloc: device %d", dev);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  SPH_CUDA(cudaStreamIsCapturing(stream, &cap), "RadixSort_noalloc: capture status");
  std::lock_guard<std::mutex> lk(g_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    SPH_CUDA(cudaGetSymbolAddress(&p, g_radix_scratch), "RadixSort_noalloc: scratch address");
    g_scratch_addr[dev] = static_cast<uint32_t*>(p);
  } else if (!g_scratch_addr[dev]) {
    return fail(SPH_ERR_STATE, "RadixSort_noalloc: first call on device %d inside a stream capture", dev);
  }
  *out = g_scratch_addr[dev];
  return SPH_OK;
}

}  // namespace

cudaStream_t stage_stream();

}  // namespace sph

extern "C" int sph_RadixSort_noalloc(sph_uint2* pData0, sph_uint2* pData1, uint32_t elements,
                                     uint32_t bits) {
  using namespace sph;
  if (elements == 0) return SPH_OK;
  if (!pData0 || !pData1) return fail(SPH_ERR_ARG, "RadixSort_noalloc: null buffer");
  if (elements > kNoAllocMaxElements)
    return fail(SPH_ERR_ARG,
                "RadixSort_noalloc: %u pairs exceed the preallocated scratch (at most %u pairs); "
                "use sph_RadixSort",
                elements, kNoAllocMaxElements);
  if (radix_scratch_words(elements) > kNoAllocWords)
    return fail(SPH_ERR_ARG, "RadixSort_noalloc: scratch too small for %u pairs", elements);
  const cudaStream_t st = stage_stream();
  uint32_t* scratch = nullptr;
  SPH_TRY(scratch_address(st, &scratch));
  return radix_sort_pairs((uint2*)pData0, (uint2*)pData1, elements, bits, scratch, st);
}
