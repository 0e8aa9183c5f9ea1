// sph_segsort.cuh -- sorting many independent segments of uint32 keys in
// place (segment k: data[start[k], start[k] + count[k])), used for the ids
// of crowded grid cells and for the per-pixel fragment lists of the
// renderer.  Three kernels:
//   k_find_cells      segments longer than `min_sort` go to `list` (up to
//                     kWarpSortMax) or `big_list`, one atomic per warp and list
//   k_sort_cells      one warp per listed segment: bitonic in shared memory
//   k_sort_big_cells  one block per big segment: bitonic in shared memory up
//                     to kBlockSortMax keys, beyond that in `scratch`
//                     (2 words per key, segment k at 2 * start[k], so the
//                     padded segments never overlap)
#pragma once
#include <cstdint>

namespace sph {
namespace {

constexpr uint32_t kWarpSortMax = 1024;   // sorted by one warp in shared memory
constexpr uint32_t kBlockSortMax = 16384; // sorted by one block in shared memory
constexpr int kSortWarps = 4;
constexpr int kBigThreads = 1024;

__device__ __forceinline__ uint32_t pow2_at_least(uint32_t n) {
  return n <= 1 ? 1u : 1u << (32 - __clz(n - 1));
}

// Bitonic sort of buf[0, m) (m a power of two) by `lanes` cooperating
// threads with index `me`; `sync` orders the stages.
template <class Sync>
__device__ __forceinline__ void bitonic(uint32_t* buf, uint32_t m, uint32_t me, uint32_t lanes,
                                        Sync sync) {
  for (uint32_t size = 2; size <= m; size <<= 1)
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t t = me; t < (m >> 1); t += lanes) {
        const uint32_t i = 2 * stride * (t / stride) + (t % stride), j = i + stride;
        const bool up = (i & size) == 0;
        const uint32_t a = buf[i], b = buf[j];
        if ((a > b) == up) {
          buf[i] = b;
          buf[j] = a;
        }
      }
      sync();
    }
}

__global__ void k_find_cells(uint32_t C, const uint32_t* __restrict__ count, uint32_t min_sort,
                             uint32_t* __restrict__ list, uint32_t* __restrict__ counters,
                             uint32_t* __restrict__ big_list) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t n = c < C ? count[c] : 0u;
  const bool mid = n > min_sort && n <= kWarpSortMax, big = n > kWarpSortMax;
  const uint32_t bm = __ballot_sync(0xffffffffu, mid), bb = __ballot_sync(0xffffffffu, big);
  uint32_t base_m = 0, base_b = 0;
  if (lane == 0) {
    if (bm) base_m = atomicAdd(counters + 0, (uint32_t)__popc(bm));
    if (bb) base_b = atomicAdd(counters + 1, (uint32_t)__popc(bb));
  }
  base_m = __shfl_sync(0xffffffffu, base_m, 0);
  base_b = __shfl_sync(0xffffffffu, base_b, 0);
  const uint32_t below = (1u << lane) - 1u;
  if (mid) list[base_m + (uint32_t)__popc(bm & below)] = c;
  if (big) big_list[base_b + (uint32_t)__popc(bb & below)] = c;
}

__global__ void __launch_bounds__(kSortWarps * 32)
k_sort_cells(const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
             uint32_t* __restrict__ slot, const uint32_t* __restrict__ list,
             const uint32_t* __restrict__ counters) {
  __shared__ uint32_t buf[kSortWarps][kWarpSortMax];
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t nl = counters[0];
  for (uint32_t q = blockIdx.x * kSortWarps + w; q < nl; q += gridDim.x * kSortWarps) {
    const uint32_t c = list[q], n = count[c], s0 = start[c], m = pow2_at_least(n);
    uint32_t* b = buf[w];
    for (uint32_t k = lane; k < m; k += 32) b[k] = k < n ? slot[s0 + k] : 0xffffffffu;
    __syncwarp();
    bitonic(b, m, lane, 32, [] { __syncwarp(); });
    for (uint32_t k = lane; k < n; k += 32) slot[s0 + k] = b[k];
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kBigThreads)
k_sort_big_cells(const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
                 uint32_t* __restrict__ slot, const uint32_t* __restrict__ big_list,
                 const uint32_t* __restrict__ big_count, uint32_t* __restrict__ scratch) {
  extern __shared__ uint32_t sbuf[];
  const uint32_t nbig = *big_count;
  for (uint32_t q = blockIdx.x; q < nbig; q += gridDim.x) {
    const uint32_t c = big_list[q], n = count[c], s0 = start[c], m = pow2_at_least(n);
    uint32_t* b = m <= kBlockSortMax ? sbuf : scratch + 2 * (size_t)s0;
    for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) b[k] = k < n ? slot[s0 + k] : 0xffffffffu;
    __syncthreads();
    if (m <= kBlockSortMax)
      bitonic(b, m, threadIdx.x, blockDim.x, [] { __syncthreads(); });
    else
      bitonic(b, m, threadIdx.x, blockDim.x, [] {
        __threadfence_block();
        __syncthreads();
      });
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) slot[s0 + k] = b[k];
    __syncthreads();
  }
}

}  // namespace
}  // namespace sph
