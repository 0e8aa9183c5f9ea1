// sph_internal.h -- host-side declarations shared by the library's
// translation units (not part of the public ABI).
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cuda_runtime.h>

#include "pibiti_sph.h"

namespace sph {

// Records the error text for sph_last_error() and returns `code`.
int fail(int code, const char* fmt, ...);
// SPH_OK, or SPH_ERR_CUDA with the CUDA error text when e != cudaSuccess.
int cuda_check(cudaError_t e, const char* what);
#define SPH_CUDA(call, what)                            \
  do {                                                  \
    int _rc = ::sph::cuda_check((call), (what));        \
    if (_rc != SPH_OK) return _rc;                      \
  } while (0)
#define SPH_TRY(expr)                                   \
  do {                                                  \
    int _rc = (expr);                                   \
    if (_rc != SPH_OK) return _rc;                      \
  } while (0)

// Checks that `p` describes a grid and kernel constants the kernels can
// run.  `fused` adds the condition the fused path's clipped neighbour walk
// needs to give the reference's results (see the definition).
int validate_params(const SimParams& p, bool fused);

// ---- exclusive scan of uint32 counts (sph_scan.cu) ----------------------
constexpr int kScanTile = 4096;  // elements per scan tile (256 threads x 16)
// Scratch words the scan needs for n elements.
size_t scan_scratch_words(size_t n);
// out[i] = sum(in[0..i)), for n < 2^32; total (if not null) gets the sum.
// `scratch` holds scan_scratch_words(n) uint32 words.
int exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                   cudaStream_t stream);
// Lists of the elements (cells) whose value (particle count) exceeds
// min_list: those up to mid_max into `mid`, the larger into `big`, the list
// lengths in counters[0] and counters[1] (order within a list unspecified).
struct ScanLists {
  uint32_t min_list, mid_max;
  uint32_t *mid, *big, *counters;
};
// exclusive_scan that also builds `lists` while it scans, in the same two
// launches.  The scan's ticket counter (scratch[0]) must be zero on entry,
// as it is after every scan (the last block clears it): the caller zeroes
// it once when it allocates the scratch.
int exclusive_scan_lists(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                         const ScanLists& lists, cudaStream_t stream);

// ---- stable LSD radix sort of (key, value) pairs (sph_scan.cu) ----------
size_t radix_scratch_words(size_t n);
// Sorts by the low `bits` bits of the key, 8 bits per pass, ping-ponging
// d0 <-> d1 as the reference's RadixSort does.
int radix_sort_pairs(uint2* d0, uint2* d1, uint32_t n, uint32_t bits, uint32_t* scratch,
                     cudaStream_t stream);

}  // namespace sph
