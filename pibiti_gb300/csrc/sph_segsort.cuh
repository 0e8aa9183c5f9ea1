// sph_segsort.cuh -- sorting many independent segments of uint32 keys
// (segment k: data[start[k], start[k] + count[k])), used for the ids of
// crowded grid cells and for the renderer's per-tile sprite lists, and
// ranking segments of distinct ids (k_rank_cells, k_rank_big_cells, below:
// the crowded cells of the step, which only need each id's rank).
// The sorting kernels:
//   k_find_cells      segments longer than `min_sort` go to `list` (up to
//                     kWarpSortMax) or `big_list`, one atomic per warp and list
//   k_sort_cells      one warp per listed segment: bitonic in registers
//                     (warp_sort_segment)
//   k_sort_big_cells  one block per big segment: bitonic in shared memory up
//                     to kBlockSortMax keys, beyond that in `scratch`
//                     (2 words per key, segment k at 2 * start[k], so the
//                     padded segments never overlap)
// The sorted keys go back in place, or, when the keys are distinct particle
// ids and `dest_of` is given, dest_of[key] = the key's sorted position
// (start[k] + rank) is written instead, which is all the cell placement
// needs.
#pragma once
#include <cstdint>

namespace sph {
namespace {

constexpr uint32_t kWarpSortMax = 1024;   // sorted by one warp in registers
constexpr uint32_t kBlockSortMax = 16384; // sorted by one block in shared memory
constexpr int kSortWarps = 4;
constexpr int kBigThreads = 1024;

__device__ __forceinline__ uint32_t pow2_at_least(uint32_t n) {
  return n <= 1 ? 1u : 1u << (32 - __clz(n - 1));
}

// Bitonic sort of buf[0, m) (m a power of two) by `lanes` cooperating
// threads with index `me`; `sync` orders the stages.  Compare-exchange t of
// a stage pairs i = 2 * stride * (t / stride) + t % stride with i + stride;
// stride is a power of two, so i = 2t - (t & (stride - 1)).
template <class Sync>
__device__ __forceinline__ void bitonic(uint32_t* buf, uint32_t m, uint32_t me, uint32_t lanes,
                                        Sync sync) {
  for (uint32_t size = 2; size <= m; size <<= 1)
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t t = me; t < (m >> 1); t += lanes) {
        const uint32_t i = 2 * t - (t & (stride - 1)), j = i + stride;
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

// One stage of stride ST < E (within each lane) and one of stride st >= E
// (lane mask st / E, by shuffles).  The stage loops stay rolled so that the
// kernel's code stays small: only the E positions of a lane are unrolled,
// which keeps v[] in registers.
template <int E, uint32_t ST>
__device__ __forceinline__ void stage_in_lane(uint32_t (&v)[E], uint32_t size, uint32_t lane) {
#pragma unroll
  for (uint32_t e = 0; e < (uint32_t)E; ++e) {
    if (e & ST) continue;
    const bool asc = ((lane * E + e) & size) == 0;
    const uint32_t a = v[e], b = v[e | ST];
    v[e] = asc ? min(a, b) : max(a, b);
    v[e | ST] = asc ? max(a, b) : min(a, b);
  }
}
template <int E>
__device__ __forceinline__ void stage_across(uint32_t (&v)[E], uint32_t size, uint32_t lm, uint32_t lane) {
  const bool lower = (lane & lm) == 0;
#pragma unroll
  for (uint32_t e = 0; e < (uint32_t)E; ++e) {
    const uint32_t o = __shfl_xor_sync(0xffffffffu, v[e], lm);
    const bool asc = ((lane * E + e) & size) == 0;
    v[e] = asc == lower ? min(v[e], o) : max(v[e], o);
  }
}

// Bitonic sort of the 32 * E keys a warp holds in registers, v[e] of lane
// `lane` at network position k = lane * E + e (the keys may be loaded in
// any order: the network sorts whatever it is given, and after it the key
// of rank k is at position k).  The partner of position k in a stage of
// stride st is k ^ st: v[e ^ st] of the same lane when st < E, the same
// e of lane lane ^ (st / E) otherwise.  Ascending where (k & size) == 0;
// the lower position of a pair keeps the minimum when ascending.  With
// E = 32 the 40 stages of stride < 32 are compare-exchanges in registers
// and only 15 are shuffles.
template <int E>
__device__ __forceinline__ void warp_bitonic(uint32_t (&v)[E], uint32_t lane) {
  constexpr uint32_t M = 32u * E;
#pragma unroll 1
  for (uint32_t size = 2; size <= M; size <<= 1) {
#pragma unroll 1
    for (uint32_t st = size >> 1; st > 0; st >>= 1) {
      if (st >= (uint32_t)E) {
        stage_across<E>(v, size, st / E, lane);
      } else {
        switch (st) {
          case 1: if constexpr (E > 1) stage_in_lane<E, 1>(v, size, lane); break;
          case 2: if constexpr (E > 2) stage_in_lane<E, 2>(v, size, lane); break;
          case 4: if constexpr (E > 4) stage_in_lane<E, 4>(v, size, lane); break;
          case 8: if constexpr (E > 8) stage_in_lane<E, 8>(v, size, lane); break;
          default: if constexpr (E > 16) stage_in_lane<E, 16>(v, size, lane); break;
        }
      }
    }
  }
}

template <int E>
__device__ __forceinline__ void warp_sort_n(uint32_t* __restrict__ data, uint32_t s0, uint32_t n,
                                            uint32_t lane, uint32_t* __restrict__ dest_of) {
  uint32_t v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {  // coalesced loads; padding sorts last
    const uint32_t k = 32u * e + lane;
    v[e] = k < n ? data[s0 + k] : 0xffffffffu;
  }
  warp_bitonic<E>(v, lane);
  if (!dest_of) __syncwarp();  // every lane has read its keys before any is written back
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const uint32_t k = lane * E + e;  // rank of v[e]
    if (k < n) {
      if (dest_of) dest_of[v[e]] = s0 + k;
      else data[s0 + k] = v[e];
    }
  }
}

// One warp sorts segment data[s0, s0 + n), n <= kWarpSortMax.
__device__ __forceinline__ void warp_sort_segment(uint32_t* __restrict__ data, uint32_t s0, uint32_t n,
                                                  uint32_t lane, uint32_t* __restrict__ dest_of) {
  if (n <= 32) warp_sort_n<1>(data, s0, n, lane, dest_of);
  else if (n <= 64) warp_sort_n<2>(data, s0, n, lane, dest_of);
  else if (n <= 128) warp_sort_n<4>(data, s0, n, lane, dest_of);
  else if (n <= 256) warp_sort_n<8>(data, s0, n, lane, dest_of);
  else if (n <= 512) warp_sort_n<16>(data, s0, n, lane, dest_of);
  else warp_sort_n<32>(data, s0, n, lane, dest_of);
}
static_assert(kWarpSortMax == 32 * 32, "warp_sort_segment covers up to 32 keys per lane");

// The same with the keys in shared memory (buf: kWarpSortMax words of this
// warp), for kernels that cannot spare the registers.
__device__ __forceinline__ void warp_sort_segment_smem(uint32_t* __restrict__ data, uint32_t s0, uint32_t n,
                                                       uint32_t lane, uint32_t* __restrict__ dest_of,
                                                       uint32_t* buf) {
  const uint32_t m = pow2_at_least(n);
  for (uint32_t k = lane; k < m; k += 32) buf[k] = k < n ? data[s0 + k] : 0xffffffffu;
  __syncwarp();
  bitonic(buf, m, lane, 32, [] { __syncwarp(); });
  for (uint32_t k = lane; k < n; k += 32) {
    if (dest_of) dest_of[buf[k]] = s0 + k;
    else data[s0 + k] = buf[k];
  }
  __syncwarp();
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
             const uint32_t* __restrict__ counters, uint32_t* __restrict__ dest_of = nullptr) {
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t nl = counters[0];
  for (uint32_t q = blockIdx.x * kSortWarps + w; q < nl; q += gridDim.x * kSortWarps) {
    const uint32_t c = list[q];
    warp_sort_segment(slot, start[c], count[c], lane, dest_of);
  }
}

// Ranks of distinct ids (particle ids of one cell) without sorting them:
// rank(id) = the number of the cell's ids below it, and dest_of[id] =
// s0 + rank.  One thread block per segment:
//   1. bucket(id) = floor((id - lo) * B / (hi - lo + 1)), B buckets, lo and
//      hi the segment's smallest and largest id; in floating point, which
//      keeps the function non-decreasing in id (every step rounds
//      monotonically), so all ids of a lower bucket are smaller;
//   2. counts per bucket (shared-memory atomics), exclusive scan of them;
//   3. each id placed into its bucket's range of a shared array;
//   4. rank = the start of its bucket + the ids of its own bucket below it.
// The work is linear in the segment as long as the buckets stay small; when
// the fullest bucket holds more than kRankBucketMax ids (ids bunched against
// an outlier) block_rank_segment returns false and the caller sorts the
// segment instead.  Bucket b's counter sits at b + b / 32, so that threads
// reading runs of consecutive counters meet few bank conflicts.
constexpr uint32_t kRankBucketMax = 32;
constexpr uint32_t kRankThreads = 256, kRankBuckets = 1024;  // cells of up to kWarpSortMax ids
constexpr uint32_t kBigRankBuckets = 4096;                   // cells of up to kBlockSortMax ids
__host__ __device__ constexpr uint32_t rank_padded(uint32_t buckets) { return buckets + buckets / 32; }
__device__ __forceinline__ uint32_t rank_slot(uint32_t b) { return b + (b >> 5); }

// Block-wide reductions and exclusive scan (blockDim.x a multiple of 32, at
// most 1024); `red` holds 32 words, and each call ends with a barrier.
__device__ __forceinline__ uint32_t block_min_max(uint32_t v, bool is_max, uint32_t* red) {
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = is_max ? __reduce_max_sync(0xffffffffu, v) : __reduce_min_sync(0xffffffffu, v);
  if (lane == 0) red[w] = v;
  __syncthreads();
  uint32_t x = lane < nw ? red[lane] : (is_max ? 0u : 0xffffffffu);
  x = is_max ? __reduce_max_sync(0xffffffffu, x) : __reduce_min_sync(0xffffffffu, x);
  __syncthreads();
  return x;
}
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* red) {
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if ((int)lane >= o) x += y;
  }
  if (lane == 31) red[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < nw ? red[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if ((int)lane >= o) t += y;
    }
    if (lane < nw) red[lane] = t;  // inclusive prefixes of the warps' totals
  }
  __syncthreads();
  const uint32_t before = w ? red[w - 1] : 0u;
  __syncthreads();
  return before + x - v;
}

// hist: rank_padded(kB) words, tmp: >= n words, red: 32 words.  Uniform
// over the block; false when a bucket is too full (nothing written then).
template <uint32_t kB>
__device__ bool block_rank_segment(const uint32_t* __restrict__ slot, uint32_t s0, uint32_t n,
                                   uint32_t* __restrict__ dest_of, uint32_t* hist, uint32_t* tmp,
                                   uint32_t* red) {
  const uint32_t t = threadIdx.x, T = blockDim.x, per = kB / T;  // buckets a thread scans
  uint32_t lo = 0xffffffffu, hi = 0u;
  for (uint32_t k = t; k < n; k += T) {
    const uint32_t id = slot[s0 + k];
    lo = min(lo, id);
    hi = max(hi, id);
  }
  lo = block_min_max(lo, false, red);
  hi = block_min_max(hi, true, red);
  const float scale = (float)kB / ((float)(hi - lo) + 1.f);
  auto bucket = [&](uint32_t id) { return min((uint32_t)((float)(id - lo) * scale), kB - 1u); };
  for (uint32_t k = t; k < rank_padded(kB); k += T) hist[k] = 0u;
  __syncthreads();
  for (uint32_t k = t; k < n; k += T) atomicAdd(&hist[rank_slot(bucket(slot[s0 + k]))], 1u);
  __syncthreads();
  uint32_t sum = 0u, most = 0u;
  for (uint32_t j = 0; j < per; ++j) {
    const uint32_t c = hist[rank_slot(t * per + j)];
    sum += c;
    most = max(most, c);
  }
  if (block_min_max(most, true, red) > kRankBucketMax) return false;
  uint32_t run = block_excl_scan(sum, red);
  for (uint32_t j = 0; j < per; ++j) {
    const uint32_t c = hist[rank_slot(t * per + j)];
    hist[rank_slot(t * per + j)] = run;
    run += c;
  }
  __syncthreads();
  // into the buckets' ranges; afterwards hist[bucket b] = the end of b
  for (uint32_t k = t; k < n; k += T) {
    const uint32_t id = slot[s0 + k];
    tmp[atomicAdd(&hist[rank_slot(bucket(id))], 1u)] = id;
  }
  __syncthreads();
  for (uint32_t k = t; k < n; k += T) {
    const uint32_t id = slot[s0 + k], b = bucket(id);
    const uint32_t b0 = b ? hist[rank_slot(b - 1u)] : 0u, b1 = hist[rank_slot(b)];
    uint32_t r = b0;
    for (uint32_t u = b0; u < b1; ++u) r += tmp[u] < id;
    dest_of[id] = s0 + r;
  }
  __syncthreads();  // hist and tmp are reused by the next segment
  return true;
}

// Bitonic sort of one segment by the block, in `buf` (pow2_at_least(n)
// words of shared memory) or, for larger segments, in `scratch` (2 words
// per key at 2 * s0, so padded segments never overlap).
__device__ __forceinline__ void block_sort_segment(uint32_t* __restrict__ slot, uint32_t s0, uint32_t n,
                                                   uint32_t* buf, uint32_t buf_words, uint32_t* __restrict__ scratch,
                                                   uint32_t* __restrict__ dest_of) {
  const uint32_t m = pow2_at_least(n);
  uint32_t* b = m <= buf_words ? buf : scratch + 2 * (size_t)s0;
  for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) b[k] = k < n ? slot[s0 + k] : 0xffffffffu;
  __syncthreads();
  if (m <= buf_words)
    bitonic(b, m, threadIdx.x, blockDim.x, [] { __syncthreads(); });
  else
    bitonic(b, m, threadIdx.x, blockDim.x, [] {
      __threadfence_block();
      __syncthreads();
    });
  for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
    if (dest_of) dest_of[b[k]] = s0 + k;
    else slot[s0 + k] = b[k];
  }
  __syncthreads();
}

// The listed cells of up to kWarpSortMax ids: ranked by buckets, or sorted
// by the block when their ids bunch.
__global__ void __launch_bounds__(kRankThreads)
k_rank_cells(const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
             uint32_t* __restrict__ slot, const uint32_t* __restrict__ list,
             const uint32_t* __restrict__ counters, uint32_t* __restrict__ dest_of) {
  __shared__ uint32_t hist[rank_padded(kRankBuckets)], tmp[kWarpSortMax], red[32];
  const uint32_t nl = counters[0];
  for (uint32_t q = blockIdx.x; q < nl; q += gridDim.x) {
    const uint32_t c = list[q], s0 = start[c], n = count[c];
    if (!block_rank_segment<kRankBuckets>(slot, s0, n, dest_of, hist, tmp, red))
      block_sort_segment(slot, s0, n, tmp, kWarpSortMax, nullptr, dest_of);
  }
}

// The listed cells above kWarpSortMax ids: ranked by buckets up to
// kBlockSortMax ids, sorted otherwise (in shared memory up to kBlockSortMax,
// through `scratch` beyond).  Dynamic shared memory: kBigRankSmem bytes.
constexpr size_t kBigRankSmem = (kBlockSortMax + rank_padded(kBigRankBuckets) + 32) * sizeof(uint32_t);
__global__ void __launch_bounds__(kBigThreads)
k_rank_big_cells(const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
                 uint32_t* __restrict__ slot, const uint32_t* __restrict__ big_list,
                 const uint32_t* __restrict__ big_count, uint32_t* __restrict__ scratch,
                 uint32_t* __restrict__ dest_of) {
  extern __shared__ uint32_t sbuf[];
  uint32_t* tmp = sbuf;
  uint32_t* hist = sbuf + kBlockSortMax;
  uint32_t* red = hist + rank_padded(kBigRankBuckets);
  const uint32_t nbig = *big_count;
  for (uint32_t q = blockIdx.x; q < nbig; q += gridDim.x) {
    const uint32_t c = big_list[q], n = count[c], s0 = start[c];
    if (n <= kBlockSortMax && block_rank_segment<kBigRankBuckets>(slot, s0, n, dest_of, hist, tmp, red))
      continue;
    block_sort_segment(slot, s0, n, tmp, kBlockSortMax, scratch, dest_of);
  }
}
static_assert(kRankBuckets % kRankThreads == 0 && kBigRankBuckets % kBigThreads == 0, "buckets per thread");

__global__ void __launch_bounds__(kBigThreads)
k_sort_big_cells(const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
                 uint32_t* __restrict__ slot, const uint32_t* __restrict__ big_list,
                 const uint32_t* __restrict__ big_count, uint32_t* __restrict__ scratch,
                 uint32_t* __restrict__ dest_of = nullptr) {
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
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
      if (dest_of) dest_of[b[k]] = s0 + k;
      else slot[s0 + k] = b[k];
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace sph
