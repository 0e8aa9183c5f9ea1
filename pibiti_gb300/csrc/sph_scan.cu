// sph_scan.cu -- exclusive scan of uint32 counts and a stable LSD radix sort
// of (key, value) pairs.
//
// Scan: two launches.  The first sums each 4096-element tile and the block
// that finishes last (an atomic ticket, no waiting) scans the tile sums; the
// second scans each tile and adds its tile's prefix.  Nothing spins.
//
// Radix sort (the stable sort RadixSort performs, radixsort_kernel.cu:
// 70-472): per 8-bit digit pass, a per-tile digit histogram (digit-major),
// the exclusive scan above over it, and a scatter that ranks the items of a
// tile in index order (rounds of 256 items, warp-level match_any for ranks
// within a round, per-warp digit counts in shared memory for ranks across
// warps), so equal digits keep their input order.
#include <cuda_runtime.h>

#include "sph_internal.h"

namespace sph {
namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = kScanTile / kThreads;  // 16
static_assert(kPerThread == 16, "tile layout");

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot,
                                                         uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kThreads / 32 ? warp_tot[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kThreads / 32) warp_tot[lane] = w;  // inclusive warp prefixes
  }
  __syncthreads();
  const uint32_t before = warp == 0 ? 0u : warp_tot[warp - 1];
  *total = warp_tot[kThreads / 32 - 1];
  __syncthreads();  // warp_tot is reused by the caller's next scan
  return before + x - v;
}

// Loads the 16 consecutive elements thread t owns in a tile.
__device__ __forceinline__ void load16(const uint32_t* in, uint32_t n, size_t first, uint32_t v[16]) {
  if (first + 16 <= n) {
    const uint4* q = reinterpret_cast<const uint4*>(in + first);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint4 a = q[k];
      v[4 * k] = a.x;
      v[4 * k + 1] = a.y;
      v[4 * k + 2] = a.z;
      v[4 * k + 3] = a.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = first + k < n ? in[first + k] : 0u;
  }
}

__global__ void __launch_bounds__(kThreads)
scan_tile_sums(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ counter,
               uint32_t* __restrict__ tile_sum, uint32_t tiles, uint32_t* __restrict__ list_counters) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t ticket;
  const size_t first = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kPerThread;
  uint32_t v[16];
  load16(in, n, first, v);
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) s += v[k];
  uint32_t total;
  block_exclusive_scan(s, warp_tot, &total);
  if (threadIdx.x == 0) {
    tile_sum[blockIdx.x] = total;
    __threadfence();
    ticket = atomicAdd(counter, 1u);
  }
  __syncthreads();
  if (ticket != tiles - 1) return;
  // Last block: every tile sum is visible; scan them in place.
  __threadfence();
  uint32_t carry = 0;
  for (uint32_t c = 0; c < tiles; c += kThreads) {
    const uint32_t i = c + threadIdx.x;
    const uint32_t x = i < tiles ? __ldcg(tile_sum + i) : 0u;
    uint32_t t;
    const uint32_t e = block_exclusive_scan(x, warp_tot, &t);
    if (i < tiles) tile_sum[i] = carry + e;
    carry += t;
  }
  if (threadIdx.x == 0) {
    *counter = 0;  // ready for the next scan
    if (list_counters) list_counters[0] = list_counters[1] = 0;  // filled by scan_tiles
  }
}

__global__ void __launch_bounds__(kThreads)
scan_tiles(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint32_t n,
           const uint32_t* __restrict__ tile_sum, ScanLists lists) {
  __shared__ uint32_t warp_tot[32];
  const size_t first = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kPerThread;
  uint32_t v[16];
  load16(in, n, first, v);
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) s += v[k];
  uint32_t total;
  uint32_t run = block_exclusive_scan(s, warp_tot, &total) + __ldcg(tile_sum + blockIdx.x);
  uint32_t o[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    o[k] = run;
    run += v[k];
  }
  if (first + 16 <= n) {
    uint4* q = reinterpret_cast<uint4*>(out + first);
#pragma unroll
    for (int k = 0; k < 4; ++k) q[k] = make_uint4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
  } else {
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (first + k < n) out[first + k] = o[k];
  }
  if (lists.counters) {
    // the elements above min_list: the block's counts of each kind scanned
    // together (mid in the low 16 bits, big in the high: at most 4096 each),
    // one atomic per list and block, then each thread writes its own
    uint32_t nm = 0, nb = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      nm += v[k] > lists.min_list && v[k] <= lists.mid_max;
      nb += v[k] > lists.mid_max;
    }
    uint32_t tot;
    const uint32_t pre = block_exclusive_scan(nm | (nb << 16), warp_tot, &tot);
    __shared__ uint32_t base_m, base_b;
    if (threadIdx.x == 0) {
      base_m = (tot & 0xFFFFu) ? atomicAdd(lists.counters + 0, tot & 0xFFFFu) : 0u;
      base_b = (tot >> 16) ? atomicAdd(lists.counters + 1, tot >> 16) : 0u;
    }
    __syncthreads();
    uint32_t om = base_m + (pre & 0xFFFFu), ob = base_b + (pre >> 16);
    if (nm | nb) {
#pragma unroll 1
      for (int k = 0; k < 16; ++k) {
        const uint32_t e = (uint32_t)(first + k);
        if (v[k] > lists.mid_max) lists.big[ob++] = e;
        else if (v[k] > lists.min_list) lists.mid[om++] = e;
      }
    }
  }
}

// ---- radix sort ---------------------------------------------------------

__global__ void __launch_bounds__(kThreads)
radix_hist(const uint2* __restrict__ src, uint32_t n, uint32_t shift, uint32_t* __restrict__ hist,
           uint32_t tiles) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * kScanTile;
#pragma unroll 4
  for (int k = 0; k < kPerThread; ++k) {
    const size_t i = base + (size_t)k * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(src[i].x >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * tiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(kThreads)
radix_scatter(const uint2* __restrict__ src, uint2* __restrict__ dst, uint32_t n, uint32_t shift,
              const uint32_t* __restrict__ offs, uint32_t tiles) {
  constexpr int kWarps = kThreads / 32;
  __shared__ uint32_t base[256];
  __shared__ uint32_t wcnt[kWarps][256];
  const int t = threadIdx.x, warp = t >> 5;
  base[t] = offs[(size_t)t * tiles + blockIdx.x];
#pragma unroll
  for (int w = 0; w < kWarps; ++w) wcnt[w][t] = 0;
  __syncthreads();
  const size_t tile0 = (size_t)blockIdx.x * kScanTile;
  for (int r = 0; r < kPerThread; ++r) {
    const size_t i = tile0 + (size_t)r * kThreads + t;
    const bool valid = i < n;
    uint2 kv = make_uint2(0u, 0u);
    uint32_t d = 256u;  // no digit
    if (valid) {
      kv = src[i];
      d = (kv.x >> shift) & 0xffu;
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & lanemask_lt());
    if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t pos = base[d] + rank;
      for (int w = 0; w < warp; ++w) pos += wcnt[w][d];
      dst[pos] = kv;
    }
    __syncthreads();
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      s += wcnt[w][t];
      wcnt[w][t] = 0;
    }
    base[t] += s;
    __syncthreads();
  }
}

inline uint32_t tiles_for(size_t n) { return (uint32_t)((n + kScanTile - 1) / kScanTile); }

}  // namespace

size_t scan_scratch_words(size_t n) { return 1 + tiles_for(n) + 3; }

int exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                   cudaStream_t stream) {
  if (n == 0) return SPH_OK;
  const uint32_t tiles = tiles_for(n);
  uint32_t* counter = scratch;
  uint32_t* tile_sum = scratch + 1;
  SPH_CUDA(cudaMemsetAsync(counter, 0, sizeof(uint32_t), stream), "scan counter reset");
  scan_tile_sums<<<tiles, kThreads, 0, stream>>>(in, n, counter, tile_sum, tiles, nullptr);
  scan_tiles<<<tiles, kThreads, 0, stream>>>(in, out, n, tile_sum, ScanLists{0, 0, nullptr, nullptr, nullptr});
  return cuda_check(cudaGetLastError(), "scan kernels");
}

int exclusive_scan_lists(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                         const ScanLists& lists, cudaStream_t stream) {
  if (n == 0) return SPH_OK;
  const uint32_t tiles = tiles_for(n);
  scan_tile_sums<<<tiles, kThreads, 0, stream>>>(in, n, scratch, scratch + 1, tiles, lists.counters);
  scan_tiles<<<tiles, kThreads, 0, stream>>>(in, out, n, scratch + 1, lists);
  return cuda_check(cudaGetLastError(), "scan kernels");
}

size_t radix_scratch_words(size_t n) {
  const size_t h = (size_t)256 * tiles_for(n);
  return 2 * h + scan_scratch_words(h);
}

int radix_sort_pairs(uint2* d0, uint2* d1, uint32_t n, uint32_t bits, uint32_t* scratch,
                     cudaStream_t stream) {
  if (n == 0 || bits == 0) return SPH_OK;
  const uint32_t tiles = tiles_for(n);
  const size_t h = (size_t)256 * tiles;
  if (h >= 0xffffffffull) return fail(SPH_ERR_ARG, "RadixSort: %u elements is too many", n);
  uint32_t* hist = scratch;
  uint32_t* offs = scratch + h;
  uint32_t* scan_tmp = scratch + 2 * h;
  uint2* src = d0;
  uint2* dst = d1;
  for (uint32_t shift = 0; shift < bits && shift < 32; shift += 8) {
    radix_hist<<<tiles, kThreads, 0, stream>>>(src, n, shift, hist, tiles);
    SPH_TRY(exclusive_scan(hist, offs, (uint32_t)h, scan_tmp, stream));
    radix_scatter<<<tiles, kThreads, 0, stream>>>(src, dst, n, shift, offs, tiles);
    SPH_CUDA(cudaGetLastError(), "radix sort kernels");
    uint2* t = src;
    src = dst;
    dst = t;
  }
  return SPH_OK;
}

}  // namespace sph
