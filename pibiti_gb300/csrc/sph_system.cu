// sph_system.cu -- the system handle: whole SPH steps with fused kernels,
// for one scene or for many independent scenes at once.
//
// Layout in HBM (N particles, C cells, over all scenes):
//   pos[2], vel[2]  float4[N]   particle state, kept in the sorted order of
//                               the previous step (not the original order)
//   id[2]           uint32[N]   original index of each stored particle
//   key, rank       uint32[N]   cell of each particle, its arrival rank there
//   slot            uint32[N]   original indices scattered into their cells
//   count, start    uint32[C]   particles per cell and first sorted index
//   dens, pres      float[N]    of the last step, sorted order
// Scenes own contiguous particle ranges and contiguous cell ranges; a
// particle's cell key is (scene cell offset + local hash), so one counting
// sort orders every scene at once and keeps each scene inside its range.
//
// One step (cSPH::Update, SPH_Update.cpp:12-81):
//   k_integrate_count  integrate each particle (in registers), find its cell,
//                      take a rank in the cell with one atomic per warp group
//   exclusive scan     count -> start, and the lists of the cells with
//                      more than 32 particles
//   k_scatter_ids      slot[start + rank] = original index
//   k_rank_cells,      each listed cell's ids ranked by buckets (a block per
//   k_rank_big_cells   cell; sorted instead where they bunch), the latter for
//                      cells above 1024 ids, on a side stream
//   k_place            stable position inside the cell = number of smaller
//                      original indices there (the reference's sort is
//                      stable on original order); integrate again and write
//                      the particle there
//   k_density          27-cell poly6 sum (Kernel_Cell.cui:142-199)
//   k_force            27-cell spiky + viscosity, collider, accelerators;
//                      the new velocity is written in sorted order
// so the sorted order (hash, original index) equals the reference's.
#include <climits>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include <cuda_bf16.h>

#include "sph_device.cuh"
#include "sph_segsort.cuh"
#include "sph_internal.h"

namespace sph {
namespace {

struct __align__(16) SceneDesc {
  SimParams p;
  uint32_t p_off, p_cnt, c_off, c_cnt;
  float inv_cell[3];  // 1 / cellSize (rounded; for scheduling keys only)
};

constexpr int kBlock = 256;
inline unsigned grid_for(size_t n, int block) { return (unsigned)((n + block - 1) / block); }

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// A read of data that stays read-only for the whole kernel (kNC: through the
// non-coherent path) or of data other blocks of the same (persistent)
// kernel write between its stages (a plain load, ordered by the barrier).
template <bool kNC, class T>
__device__ __forceinline__ T ld(const T* p) {
  if constexpr (kNC) return __ldg(p);
  else return *p;
}

// Scene holding element i of a concatenation with offsets off[0..S].
__device__ __forceinline__ int scene_of(const uint32_t* __restrict__ off, int S, uint32_t i) {
  int lo = 0, hi = S - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(off + mid) <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Integrate particle i, find its cell and take a rank in it with one
// atomicAdd per group of lanes sharing the cell.  Called by all 32 lanes
// of a warp for consecutive i (i >= N: the lane takes part but does nothing).
__device__ __forceinline__ void integrate_count_item(const SceneDesc* __restrict__ sc,
                                                     const uint32_t* __restrict__ poff, int S,
                                                     uint32_t N, const float4* __restrict__ pos,
                                                     const float4* __restrict__ vel,
                                                     uint32_t* __restrict__ key,
                                                     uint32_t* __restrict__ rank,
                                                     uint32_t* __restrict__ count,
                                                     uint32_t* __restrict__ flags, uint32_t i) {
  const bool valid = i < N;
  uint32_t gcell = 0xffffffffu;
  if (valid) {
    const SceneDesc& d = sc[S == 1 ? 0 : scene_of(poff, S, i)];
    const float4 x4 = pos[i], v4 = vel[i];
    float3 x = make_float3(x4.x, x4.y, x4.z), v = make_float3(v4.x, v4.y, v4.z);
    integrate(d.p, x, v);
    if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) atomicOr(flags, 2u);
    gcell = d.c_off + cell_of(d.p, grid_pos(d.p, make_float4(x.x, x.y, x.z, 0.f)));
  }
  const uint32_t peers = __match_any_sync(0xffffffffu, gcell);
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (valid && (int)(threadIdx.x & 31) == leader) base = atomicAdd(count + gcell, __popc(peers));
  base = __shfl_sync(peers, base, leader);
  if (valid) {
    key[i] = gcell;
    rank[i] = base + __popc(peers & lanemask_lt());
  }
}

__global__ void __launch_bounds__(kBlock)
k_integrate_count(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S,
                  uint32_t N, const float4* __restrict__ pos, const float4* __restrict__ vel,
                  uint32_t* __restrict__ key, uint32_t* __restrict__ rank,
                  uint32_t* __restrict__ count, uint32_t* __restrict__ flags) {
  integrate_count_item(sc, poff, S, N, pos, vel, key, rank, count, flags,
                       blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void __launch_bounds__(kBlock)
k_scatter_ids(uint32_t N, const uint32_t* __restrict__ key, const uint32_t* __restrict__ rank,
              const uint32_t* __restrict__ id, const uint32_t* __restrict__ start,
              uint32_t* __restrict__ slot) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  slot[start[key[i]] + rank[i]] = id[i];
}

// Cells with more than kLinearRank particles get their id segment of
// `slot` sorted (sph_segsort.cuh), which writes each id's sorted position to
// dest_of[id] for k_place; in smaller cells k_place counts the smaller ids
// linearly.  Sorting is by original index, the order the reference's stable
// sort gives within a cell.
constexpr uint32_t kLinearRank = 32;

__device__ __forceinline__ void place_item(const SceneDesc* __restrict__ sc,
                                           const uint32_t* __restrict__ poff, int S, uint32_t N,
                                           const float4* __restrict__ pos,
                                           const float4* __restrict__ vel,
                                           const uint32_t* __restrict__ id,
                                           const uint32_t* __restrict__ key,
                                           const uint32_t* __restrict__ start,
                                           const uint32_t* __restrict__ count,
                                           const uint32_t* __restrict__ slot,
                                           const uint32_t* __restrict__ dest_of,
                                           float4* __restrict__ pos_out,
                                           float4* __restrict__ vel_out,
                                           uint32_t* __restrict__ id_out,
                                           float4* __restrict__ vel_start, uint32_t i) {
  const uint32_t c = key[i], s0 = start[c], n = count[c], me = id[i];
  uint32_t dest;
  if (n <= kLinearRank) {
    uint32_t r = 0;
    for (uint32_t j = s0; j < s0 + n; ++j) r += slot[j] < me;
    dest = s0 + r;
  } else {
    dest = dest_of[me];  // written by the cell's sort
  }
  const SceneDesc& d = sc[S == 1 ? 0 : scene_of(poff, S, i)];
  const float4 x4 = pos[i], v4 = vel[i];
  float3 x = make_float3(x4.x, x4.y, x4.z), v = make_float3(v4.x, v4.y, v4.z);
  integrate(d.p, x, v);
  pos_out[dest] = make_float4(x.x, x.y, x.z, x4.w);
  vel_out[dest] = make_float4(v.x, v.y, v.z, v4.w);
  id_out[dest] = me;
  if (vel_start) vel_start[dest] = v4;  // the velocity before gravity and the walls
}

__global__ void __launch_bounds__(kBlock)
k_place(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
        const float4* __restrict__ pos, const float4* __restrict__ vel,
        const uint32_t* __restrict__ id, const uint32_t* __restrict__ key,
        const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
        const uint32_t* __restrict__ slot, const uint32_t* __restrict__ dest_of,
        float4* __restrict__ pos_out, float4* __restrict__ vel_out, uint32_t* __restrict__ id_out,
        float4* __restrict__ vel_start = nullptr) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  place_item(sc, poff, S, N, pos, vel, id, key, start, count, slot, dest_of, pos_out, vel_out, id_out,
             vel_start, i);
}

// Launch shapes of the two walks: threads per block and the form of each
// walk.  Density: 0 = one particle per thread over global memory
// (density_item), 1 = candidates staged in shared memory (k_density_tile),
// 2 = staged as interleaved pairs (k_density_pairs).  Force: 0 = global
// memory, row masks two bits at a time (force_item), 1 = staged
// (k_force_tile), 2 = global memory, one cell field at a time
// (k_force_fields), 3 = global memory, pair terms evaluated by the whole
// warp row by row (k_force_coop; 64 or 128 threads).  The global forms run 64, 128 or 256 threads at 64
// registers (the featured force pass: 7/8 of those blocks, 72 registers).
// sph_autotune picks one per handle by timing them on the handle's own
// scenes; without neighbour masks (maxParInCell > 16) every shape walks
// global memory, one particle per thread, unmasked.
struct WalkShape {
  int threads, dens, force;
};
constexpr int kWalkShapes = 11;
constexpr WalkShape kShapes[kWalkShapes] = {
    {64, 0, 0}, {128, 0, 0}, {256, 0, 0}, {128, 1, 1}, {128, 2, 2}, {256, 2, 2},
    {128, 2, 0}, {128, 0, 2}, {64, 2, 2}, {128, 2, 3}, {64, 2, 3}};
constexpr uint32_t kTileDensSlots = 2048, kTileForceSlots = 1536;  // shape 3
constexpr uint32_t kPairs64 = 512, kPairs128 = 896, kPairs256 = 1792;  // k_density_pairs
constexpr int kDefaultShape = 4;
static_assert(kWalkShapes == SPH_WALK_SHAPES, "walk shapes in pibiti_sph.h");

// Neighbour masks: with maxParInCell <= 16, the density pass records for
// each particle and each of the 9 neighbour rows (dz, dy) one 64-bit mask
// over the row's candidates: a 16-bit field per x offset (dx = -1 in bits
// 32-47, dx = 0 in bits 16-31, dx = +1 in bits 0-15), and in a field, bit
// 15 - k for the cell's k-th candidate (its k-th particle, k < maxParInCell).
// Bit set = squared distance below ForceConsts::h2_out (or NaN).  The highest
// set bit is the first candidate in walk order, so the force pass visits
// exactly those candidates, in the same order, by repeatedly taking the
// highest set bit; its sums are unchanged, and it skips the rest, which the
// density pass has shown contribute nothing.  The layout does not depend on
// how many particles the cells hold, so a walk that stages the candidates
// somewhere else reads the same masks.
constexpr int kRows = 9;
constexpr uint32_t kMaskMaxPerCell = 16;
#ifndef SPH_WALK_MASKS
#define SPH_WALK_MASKS 1  // 0: no mask buffer (saves 72 B per particle)
#endif

// Field (dx + 1) and candidate index of mask bit b.
__device__ __forceinline__ int mask_field(int b) { return 2 - (b >> 4); }
__device__ __forceinline__ uint32_t mask_cand(int b) { return (uint32_t)(15 - (b & 15)); }
// The field of a cell whose candidate k is bit k of `m` (k < 16).
__device__ __forceinline__ unsigned long long mask_place(uint32_t m, int field) {
  return (unsigned long long)(__brev(m) >> 16) << (16 * (2 - field));
}

__device__ __forceinline__ float h2_out_of(const SimParams& p) {
  return __int_as_float(__float_as_int(__fmul_rn(p.h, p.h)) + 2);
}

template <bool kMask, bool kNC = true>
__device__ __forceinline__ void density_item(const SceneDesc* __restrict__ sc,
                                             const uint32_t* __restrict__ poff, int S, uint32_t N,
                                             const float4* __restrict__ pos,
                                             const uint32_t* __restrict__ start,
                                             const uint32_t* __restrict__ count,
                                             float* __restrict__ dens_out,
                                             float* __restrict__ pres_out,
                                             float2* __restrict__ dp_out,
                                             unsigned long long* __restrict__ masks,
                                             uint32_t* __restrict__ flags, uint32_t i) {
  const SceneDesc& d = sc[S == 1 ? 0 : scene_of(poff, S, i)];
  const SimParams& p = d.p;
  const float4 xi = pos[i];
  const float h2 = p.h2, h2_out = h2_out_of(p);
  const int3 g = grid_pos(p, xi);
  const int gx = (int)p.gridSize.x, gy = (int)p.gridSize.y, gz = (int)p.gridSize.z;
  const int cx = min(max(g.x, 0), gx - 1), cy = min(max(g.y, 0), gy - 1), cz = min(max(g.z, 0), gz - 1);
  const uint32_t maxpc = p.maxParInCell;
  const int x0 = max(cx - 1, 0), x1 = min(cx + 1, gx - 1);
  float sum = 0.f;
  bool trunc = false;
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    const int z = cz + r / 3 - 1, y = cy + r % 3 - 1;
    unsigned long long rowmask = 0;
    if (z >= 0 && z < gz && y >= 0 && y < gy) {
      const uint32_t row = d.c_off + (uint32_t)(z * (int)p.gridSize_yx + y * gx);
#pragma unroll 1
      for (int x = x0; x <= x1; ++x) {
        const uint32_t c = row + (uint32_t)x;
        uint32_t n = ld<kNC>(count + c);
        if (n > maxpc) {
          trunc = true;
          n = maxpc;
        }
        const uint32_t s0 = ld<kNC>(start + c);
        float cell = 0.f;
        uint32_t m = 0;
        // only the particle's own cell holds i
        const uint32_t self = (r == 4 && x == cx) ? i - s0 : 0xffffffffu;
        auto cand = [&](uint32_t k) {
          const float4 xj = ld<kNC>(pos + s0 + k);
          const float dx = __fsub_rn(xi.x, xj.x), dy = __fsub_rn(xi.y, xj.y), dz = __fsub_rn(xi.z, xj.z);
          const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
          if (r2 < h2) {
            const float cc = __fsub_rn(h2, r2);
            cell = __fmaf_rn(__fmul_rn(cc, cc), cc, cell);
          }
          if (kMask && !(r2 >= h2_out)) m |= 1u << k;
        };
        if (self < n) {
#pragma unroll 4
          for (uint32_t k = 0; k < self; ++k) cand(k);
#pragma unroll 4
          for (uint32_t k = self + 1; k < n; ++k) cand(k);
        } else {
#pragma unroll 4
          for (uint32_t k = 0; k < n; ++k) cand(k);
        }
        sum = __fadd_rn(sum, cell);
        if (kMask) rowmask |= mask_place(m, x - cx + 1);
      }
    }
    if (kMask) masks[(size_t)r * N + i] = rowmask;
  }
  if (trunc) atomicOr(flags, 1u);
  const float dens = __fmul_rn(__fmul_rn(sum, p.Poly6Kern), p.particleMass);
  const float pres = __fmul_rn(__fsub_rn(dens, p.restDensity), p.stiffness);
  dens_out[i] = dens;
  pres_out[i] = pres;
  dp_out[i] = make_float2(__frcp_rn(dens), pres);  // the force pass's per-neighbour record
}

template <bool kMask, int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
k_density(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
          const float4* __restrict__ pos, const uint32_t* __restrict__ start,
          const uint32_t* __restrict__ count, float* __restrict__ dens_out,
          float* __restrict__ pres_out, float2* __restrict__ dp_out,
          unsigned long long* __restrict__ masks, uint32_t* __restrict__ flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  density_item<kMask>(sc, poff, S, N, pos, start, count, dens_out, pres_out, dp_out, masks, flags, i);
}

// Learned-corrector features of particle i (SPH_MLP_IN = 16), from the
// neighbours the force pass visits with r < h, weight w = ((h - r)/h)^2:
//   0 rho/rho0 - 1            1 p / (rho0 g h)          2 neighbours / 64
//   3 dt/h sum w (v_j - v_i).(x_i - x_j)/r               (velocity divergence)
//   4-6 dt/h sum w (v_j - v_i) / sum w                   (relative velocity moment)
//   7-9 sum w (x_j - x_i)/h / sum w                      (position moment)
//   10-12 SPH velocity increment / (g dt)
//   13-15 soft-wall velocity increment boundary() gives at the current
//         position and velocity, / (g dt)   (the stiff wall term is where
//         a 4x step departs most from four small ones)
// Written raw (FP32) and/or standardised ((f - mean) * inv_std) in BF16.
struct FeatAcc {
  float sw = 0.f, n = 0.f, div = 0.f, rv[3] = {0.f, 0.f, 0.f}, rx[3] = {0.f, 0.f, 0.f};
};
struct FeatOut {
  float* raw;               // N x 16 FP32 or null
  uint16_t* norm;           // N x 16 BF16 or null
  const float* stats;       // mean[16], inv_std[16]
};

// One pair's contribution to the learned step's features (network inputs,
// BF16: approximate reciprocals suffice).
__device__ __forceinline__ void feat_add(FeatAcc& fa, const ForceConsts& k, float inv_h, float4 vi, float4 vj,
                                         float rx, float ry, float rz, float dist2) {
  const float ir = rsqrtf(fmaxf(dist2, k.minDist * k.minDist));
  const float r = fmaxf(k.minDist, dist2 * ir);
  if (r < k.h) {
    const float q = 1.f - r * inv_h, w = q * q;
    const float dvx = vj.x - vi.x, dvy = vj.y - vi.y, dvz = vj.z - vi.z;
    fa.sw += w;
    fa.n += 1.f;
    fa.div += w * (dvx * rx + dvy * ry + dvz * rz) * ir;
    fa.rv[0] += w * dvx;
    fa.rv[1] += w * dvy;
    fa.rv[2] += w * dvz;
    fa.rx[0] -= w * rx;
    fa.rx[1] -= w * ry;
    fa.rx[2] -= w * rz;
  }
}

// The 16 features of particle i from its accumulated pair sums, its SPH
// force sum F and its state, raw (FP32) and/or standardised (BF16).
__device__ __forceinline__ void feature_out(const SimParams& p, const FeatAcc& fa, float3 F, float4 xi, float4 vi,
                                            float pi, float dens_i, FeatOut fo, uint32_t i) {
  const float dt = p.timeStep, h = p.h;
  const float g = sqrtf(p.gravity.x * p.gravity.x + p.gravity.y * p.gravity.y +
                        p.gravity.z * p.gravity.z) + 1e-6f;
  const float s = __fmul_rn(p.particleMass, p.timeStep), isw = 1.f / (fa.sw + 1e-6f);
  float f[16];
  f[0] = dens_i / p.restDensity - 1.f;
  f[1] = pi / (p.restDensity * g * h);
  f[2] = fa.n * (1.f / 64.f);
  f[3] = fa.div * dt / h;
  f[4] = fa.rv[0] * isw * dt / h;
  f[5] = fa.rv[1] * isw * dt / h;
  f[6] = fa.rv[2] * isw * dt / h;
  f[7] = fa.rx[0] * isw / h;
  f[8] = fa.rx[1] * isw / h;
  f[9] = fa.rx[2] * isw / h;
  f[10] = F.x * s / (g * dt);
  f[11] = F.y * s / (g * dt);
  f[12] = F.z * s / (g * dt);
  {
    float3 bx = make_float3(xi.x, xi.y, xi.z), bv = make_float3(vi.x, vi.y, vi.z);
    boundary(p, bx, bv);
    f[13] = (bv.x - vi.x) / (g * dt);
    f[14] = (bv.y - vi.y) / (g * dt);
    f[15] = (bv.z - vi.z) / (g * dt);
  }
  if (fo.raw) {
    float4* o = reinterpret_cast<float4*>(fo.raw + (size_t)i * 16);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
  }
  if (fo.norm) {
    uint32_t u[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float a = (f[2 * q] - fo.stats[2 * q]) * fo.stats[16 + 2 * q];
      const float b = (f[2 * q + 1] - fo.stats[2 * q + 1]) * fo.stats[16 + 2 * q + 1];
      __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
      u[q] = *reinterpret_cast<uint32_t*>(&v);
    }
    uint4* o = reinterpret_cast<uint4*>(fo.norm + (size_t)i * 16);
    o[0] = make_uint4(u[0], u[1], u[2], u[3]);
    o[1] = make_uint4(u[4], u[5], u[6], u[7]);
  }
}

template <bool kMask, bool kFeat, bool kNC = true>
__device__ __forceinline__ void force_item(const SceneDesc* __restrict__ sc,
                                           const uint32_t* __restrict__ poff, int S, uint32_t N,
                                           const float4* __restrict__ pos,
                                           const float4* __restrict__ vel,
                                           const float* __restrict__ dens,
                                           const float2* __restrict__ dp,
                                           const uint32_t* __restrict__ start,
                                           const uint32_t* __restrict__ count,
                                           const unsigned long long* __restrict__ masks,
                                           float4* __restrict__ vel_out, FeatOut fo, uint32_t i) {
  const SceneDesc& d = sc[S == 1 ? 0 : scene_of(poff, S, i)];
  const SimParams& p = d.p;
  const float4 xi = pos[i], vi = vel[i];
  const float2 dpi = dp[i];
  const float inv_di = dpi.x, pi = dpi.y;
  const ForceConsts k = force_consts(p);
  const int3 g = grid_pos(p, xi);
  const int gx = (int)p.gridSize.x, gy = (int)p.gridSize.y, gz = (int)p.gridSize.z;
  const int cx = min(max(g.x, 0), gx - 1), cy = min(max(g.y, 0), gy - 1), cz = min(max(g.z, 0), gz - 1);
  const uint32_t maxpc = p.maxParInCell;
  const int x0 = max(cx - 1, 0), x1 = min(cx + 1, gx - 1);
  float3 F = make_float3(0.f, 0.f, 0.f);
  FeatAcc fa;
  const float inv_h = kFeat ? 1.f / p.h : 0.f;
  auto feat = [&](float4 vj, float rx, float ry, float rz, float dist2) {
    feat_add(fa, k, inv_h, vi, vj, rx, ry, rz, dist2);
  };
  // Pair term of candidate j (the masks already hold dist2 < h2_out):
  // returns whether r < h, with the term in f.
  auto term = [&](uint32_t j, float3& f, bool with_feat) -> bool {
    const float4 xj = ld<kNC>(pos + j);
    const float rx = __fsub_rn(xi.x, xj.x), ry = __fsub_rn(xi.y, xj.y), rz = __fsub_rn(xi.z, xj.z);
    const float dist2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmul_rn(rx, rx)));
    const float4 vj = ld<kNC>(vel + j);
    const float2 dpj = ld<kNC>(dp + j);
    const bool in = force_term(k, vi, inv_di, pi, vj, dpj.x, dpj.y, rx, ry, rz, dist2, f);
    if (kFeat && with_feat) feat(vj, rx, ry, rz, dist2);
    return in;
  };
  // Candidate j of the unmasked walk: skipped beyond h2_out before the loads.
  auto pair = [&](uint32_t j, float3& cell) {
    const float4 xj = ld<kNC>(pos + j);
    const float rx = __fsub_rn(xi.x, xj.x), ry = __fsub_rn(xi.y, xj.y), rz = __fsub_rn(xi.z, xj.z);
    const float dist2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmul_rn(rx, rx)));
    if (!(dist2 >= k.h2_out)) {
      const float4 vj = ld<kNC>(vel + j);
      const float2 dpj = ld<kNC>(dp + j);
      force_pair_near(k, vi, inv_di, pi, vj, dpj.x, dpj.y, rx, ry, rz, dist2, cell);
      if (kFeat) feat(vj, rx, ry, rz, dist2);
    }
  };
  float3 cell = make_float3(0.f, 0.f, 0.f);
  auto flush = [&]() {
    F.x = __fadd_rn(F.x, cell.x);
    F.y = __fadd_rn(F.y, cell.y);
    F.z = __fadd_rn(F.z, cell.z);
    cell = make_float3(0.f, 0.f, 0.f);
  };
  if (kMask) {
    // Row by row for all lanes together (mask and cell loads coalesced and
    // issued at the same time), then the row's set bits in walk order; the
    // cell partial sum is flushed into F when the cell changes.
#pragma unroll 1
    for (int r = 0; r < kRows; ++r) {
      const int z = cz + r / 3 - 1, y = cy + r % 3 - 1;
      if (z < 0 || z >= gz || y < 0 || y >= gy) continue;
      unsigned long long m = masks[(size_t)r * N + i];
      if (!m) continue;
      // cell starts by field (dx + 1); a field outside the grid holds no bit
      const uint32_t row = d.c_off + (uint32_t)(z * (int)p.gridSize_yx + y * gx) + (uint32_t)cx;
      const uint32_t s0 = cx > 0 ? ld<kNC>(start + (row - 1)) : 0u;
      const uint32_t s1 = ld<kNC>(start + row);
      const uint32_t s2 = cx + 1 < gx ? ld<kNC>(start + row + 1) : 0u;
      int cur = -1;
      auto index_of_bit = [&](int b, int c) {
        return (c == 0 ? s0 : (c == 1 ? s1 : s2)) + mask_cand(b);
      };
      // Two set bits per iteration: the two terms are independent (their
      // loads, square roots and divisions overlap) and are added in order.
      while (m) {
        const int ba = 63 - __clzll((long long)m);
        m ^= 1ull << ba;
        const bool two = m != 0;
        const int bb = two ? 63 - __clzll((long long)m) : ba;
        if (two) m ^= 1ull << bb;
        const int ca = mask_field(ba), cb = mask_field(bb);
        float3 fa_, fb_;
        const bool ina = term(index_of_bit(ba, ca), fa_, true);
        const bool inb = term(index_of_bit(bb, cb), fb_, two);
        if (ca != cur) {
          flush();
          cur = ca;
        }
        if (ina) {
          cell.x = __fadd_rn(cell.x, fa_.x);
          cell.y = __fadd_rn(cell.y, fa_.y);
          cell.z = __fadd_rn(cell.z, fa_.z);
        }
        if (two) {
          if (cb != cur) {
            flush();
            cur = cb;
          }
          if (inb) {
            cell.x = __fadd_rn(cell.x, fb_.x);
            cell.y = __fadd_rn(cell.y, fb_.y);
            cell.z = __fadd_rn(cell.z, fb_.z);
          }
        }
      }
      flush();
    }
  } else {
#pragma unroll 1
    for (int r = 0; r < kRows; ++r) {
      const int z = cz + r / 3 - 1, y = cy + r % 3 - 1;
      if (z < 0 || z >= gz || y < 0 || y >= gy) continue;
      const uint32_t row = d.c_off + (uint32_t)(z * (int)p.gridSize_yx + y * gx);
#pragma unroll 1
      for (int x = x0; x <= x1; ++x) {
        const uint32_t c = row + (uint32_t)x;
        const uint32_t n = min(ld<kNC>(count + c), maxpc);
        const uint32_t s0 = ld<kNC>(start + c);
#pragma unroll 4
        for (uint32_t q = 0; q < n; ++q)
          if (s0 + q != i) pair(s0 + q, cell);
        flush();
      }
    }
  }
  const float3 add = velocity_increment(p, F, xi, vi);
  vel_out[i] = make_float4(__fadd_rn(vi.x, add.x), __fadd_rn(vi.y, add.y), __fadd_rn(vi.z, add.z),
                           __fadd_rn(vi.w, 0.f));
  if (kFeat) feature_out(p, fa, F, xi, vi, pi, dens[i], fo, i);
}

// Which thread of the block runs which of its particles does not change a
// result, only how alike the lanes of a warp are: a lane's work in the
// masked walk is its neighbours row by row (rows are (z, y) offsets), and the
// warp waits for its busiest lane in every row.  Particles that sit at
// nearby z, then y, within the same cell have similar row counts, so a block
// whose particles lie in a few crowded cells hands them out in the order of
// the key (cell - the block's first cell, z and y within the cell in
// sixteenths, thread), sorted in shared memory.  At the crowded state this
// takes the lanes busy from ~59% to ~74% (a model of the walk on that state's
// masks).  A block over more than kRegroupSpan cells (small cells: little to
// gain) keeps its order and skips the sort.  The keys use the rounded
// reciprocal of the cell size: a key off by one cell only regroups worse.
constexpr uint32_t kRegroupSpan = 4;

template <int kThreads>
__device__ __forceinline__ uint32_t regrouped_particle(const SceneDesc* __restrict__ sc,
                                                       const uint32_t* __restrict__ poff, int S, uint32_t N,
                                                       const float4* __restrict__ pos) {
  static_assert(kThreads <= 256, "thread index in the key's low 8 bits");
  __shared__ uint32_t skey[kThreads];
  __shared__ uint32_t sfirst, slast;
  const uint32_t t = threadIdx.x, i0 = blockIdx.x * kThreads, i = i0 + t;
  uint32_t cell = 0, sub = 0;
  if (i < N) {
    const SceneDesc& d = sc[S == 1 ? 0 : scene_of(poff, S, i)];
    const SimParams& p = d.p;
    const float4 x = __ldg(pos + i);
    const float gx = (x.x - p.worldMin.x) * d.inv_cell[0];
    const float gy = (x.y - p.worldMin.y) * d.inv_cell[1];
    const float gz = (x.z - p.worldMin.z) * d.inv_cell[2];
    const float fx = floorf(gx), fy = floorf(gy), fz = floorf(gz);
    cell = d.c_off + cell_of(p, make_int3((int)fx, (int)fy, (int)fz));
    const uint32_t sz = (uint32_t)min(max((int)((gz - fz) * 16.f), 0), 15);
    const uint32_t sy = (uint32_t)min(max((int)((gy - fy) * 16.f), 0), 15);
    sub = (sz << 4) | sy;
  }
  const uint32_t last = min(N - 1 - i0, (uint32_t)kThreads - 1);
  if (t == 0) sfirst = cell;  // the block's first particle (always < N)
  if (t == last) slast = cell;
  __syncthreads();
  const uint32_t base = sfirst;
  if (slast - base > kRegroupSpan) return i;  // uniform over the block
  skey[t] = i < N ? (min(cell - base, 0x7FFFu) << 16) | (sub << 8) | t : 0xFFFFFFFFu;
  __syncthreads();
  bitonic(skey, kThreads, t, kThreads, [] { __syncthreads(); });
  const uint32_t k = skey[t];
  return k == 0xFFFFFFFFu ? 0xFFFFFFFFu : i0 + (k & 0xFFu);
}

template <bool kMask, int kThreads, int kMinBlocks, bool kFeat>
__global__ void __launch_bounds__(kThreads, kFeat ? kMinBlocks * 7 / 8 : kMinBlocks)
k_force(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
        const float4* __restrict__ pos, const float4* __restrict__ vel,
        const float* __restrict__ dens, const float2* __restrict__ dp,
        const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
        const unsigned long long* __restrict__ masks, float4* __restrict__ vel_out, FeatOut fo) {
  const uint32_t i = kMask ? regrouped_particle<kThreads>(sc, poff, S, N, pos)
                           : blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  force_item<kMask, kFeat>(sc, poff, S, N, pos, vel, dens, dp, start, count, masks, vel_out, fo, i);
}

#include "sph_walk_tile.cuh"

// After a coarse step of dt_c = n dt (sorted order).  Within a step,
// gravity and the wall kicks act before the drift (integrate) and the SPH
// force and colliders after it (the force pass).  With v0 the velocity the
// step started from, vs the integrated velocity the force pass started
// from and v1 its result:
//   dv_pre  = vs - v0   (gravity and walls, evaluated at the start),
//   dv_post = v1 - vs   (SPH force and colliders, evaluated at the end).
// n steps of dt sample the post-drift accelerations at t + k dt, k = 1..n,
// and the pre-drift ones at k = 0..n-1; one step of dt_c samples both once.
// For accelerations that vary linearly in time the velocity of the n fine
// steps differs by
//   jerk * ((dv_pre - dv_pre') - (dv_post - dv_post')),  jerk = (n-1)/(2n),
// (primes: the previous coarse step of the same particle, kept by original
// index in `hist`), and for constant ones the position by
//   drift * dt_c * (dv_post - dv_pre),  drift = (n-1)/(2n).
// The network's correction dv = y * out_scale * |g| * dt_c (when y is
// given) is added to the velocity and counted with dv_post in the drift.
__global__ void k_apply_correction(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff,
                                   int S, uint32_t N, const float* __restrict__ y,
                                   const float* __restrict__ out_scale, float drift, float jerk,
                                   const float4* __restrict__ vel_start,
                                   const float4* __restrict__ vel_sorted,
                                   const uint32_t* __restrict__ id, float4* __restrict__ hist,
                                   bool hist_valid, float4* __restrict__ pos,
                                   float4* __restrict__ vel) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const SimParams& p = sc[S == 1 ? 0 : scene_of(poff, S, i)].p;
  const float dt = p.timeStep;
  const float4 vs = vel_sorted[i], v0 = vel_start[i];
  float4 v = vel[i];
  const float3 post = make_float3(v.x - vs.x, v.y - vs.y, v.z - vs.z);
  const float3 pre = make_float3(vs.x - v0.x, vs.y - v0.y, vs.z - v0.z);
  if (jerk != 0.f) {
    const uint32_t me = id[i];
    if (hist_valid) {
      const float4 h = hist[me];  // previous dv_pre - dv_post
      v.x += jerk * ((pre.x - post.x) - h.x);
      v.y += jerk * ((pre.y - post.y) - h.y);
      v.z += jerk * ((pre.z - post.z) - h.z);
    }
    hist[me] = make_float4(pre.x - post.x, pre.y - post.y, pre.z - post.z, 0.f);
  }
  if (y) {
    const float g = sqrtf(p.gravity.x * p.gravity.x + p.gravity.y * p.gravity.y +
                          p.gravity.z * p.gravity.z) + 1e-6f;
    const float u = g * dt;
    v.x += y[3 * i + 0] * out_scale[0] * u;
    v.y += y[3 * i + 1] * out_scale[1] * u;
    v.z += y[3 * i + 2] * out_scale[2] * u;
  }
  vel[i] = v;
  if (drift != 0.f) {
    const float k = drift * dt;
    float4 x = pos[i];
    x.x += k * ((v.x - vs.x) - pre.x);
    x.y += k * ((v.y - vs.y) - pre.y);
    x.z += k * ((v.z - vs.z) - pre.z);
    pos[i] = x;
  }
}

// Colour and dye of the step (computeForceD's colour part, System.cu:405-546)
// for a caller that asked for them, after the force pass: clr and dye are
// in original order (the dye is read and written: it carries over between
// steps).  The velocity increment is taken as v_new - v_start; the CLR_Vel
// foam sum walks the reference's 27 wrapped cell hashes in its x-outer
// order over the same truncated cell contents.
__global__ void k_color(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S,
                        uint32_t N, const float4* __restrict__ pos,
                        const float4* __restrict__ vel_start, const float4* __restrict__ vel_new,
                        const float* __restrict__ dens, const uint32_t* __restrict__ start,
                        const uint32_t* __restrict__ count, const uint32_t* __restrict__ id,
                        float4* __restrict__ clr, float* __restrict__ dye) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const SceneDesc& d = sc[S == 1 ? 0 : scene_of(poff, S, i)];
  const SimParams& p = d.p;
  const float4 xi = pos[i], vi = vel_start[i], vn = vel_new[i];
  const float3 add = make_float3(__fsub_rn(vn.x, vi.x), __fsub_rn(vn.y, vi.y), __fsub_rn(vn.z, vi.z));
  float vdiff = 0.f;
  if (p.clrType == SPH_CLR_VEL) {
    // The reference's walk (System.cu:440-462) visits the 27 wrapped hashes
    // of the unclamped cell (calcGridHash): a hash outside the table fetches
    // cellStart 0 from the texture and stops at its first particle, whose
    // hash cannot match; an in-table hash is a cell, possibly on the other
    // side of the grid (its particles count while within the foam radius
    // of 3).  Fetches past the scene's particles return zero, whose hash 0
    // matches cell 0: an empty cell 0 yields one term with a zero
    // neighbour, a cell 0 that ends the particle list one per missing slot.
    const int3 g = grid_pos(p, xi);
    const uint32_t ns = p.numParticles;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int x = -1; x < 2; ++x)
      for (int y = -1; y < 2; ++y)
        for (int z = -1; z < 2; ++z) {
          const uint32_t gh = grid_hash_raw(p, g.x + x, g.y + y, g.z + z);
          if ((int)gh < 0 || gh >= p.numCells) continue;
          const uint32_t c = d.c_off + gh, n = __ldg(count + c);
          if (n == 0) {
            if (gh == 0) vdiff = __fadd_rn(vdiff, foam_term(xi, vi, zero, zero));
            continue;
          }
          const uint32_t s0 = __ldg(start + c), s0_local = s0 - d.p_off;
          for (uint32_t q = 0; q < p.maxParInCell; ++q) {
            if (q < n) {
              const uint32_t j = s0 + q;
              if (j != i) vdiff = __fadd_rn(vdiff, foam_term(xi, vi, __ldg(pos + j), __ldg(vel_start + j)));
            } else if (s0_local + q >= ns && gh == 0) {
              vdiff = __fadd_rn(vdiff, foam_term(xi, vi, zero, zero));
            } else {
              break;  // the next particle belongs to another cell
            }
          }
        }
  }
  const uint32_t me = id[i];
  float4 c;
  if (color_dye(p, xi, vi, dens[i], add, vdiff, dye ? dye + me : nullptr, c)) clr[me] = c;
}

// ---- buffer API kernels ---------------------------------------------------

__global__ void k_iota(uint32_t* __restrict__ a, uint32_t N) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) a[i] = i;
}

__global__ void k_set_array(float4* __restrict__ arr, const uint32_t* __restrict__ id,
                            const float4* __restrict__ src, uint32_t start, uint32_t cnt,
                            uint32_t N) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const uint32_t o = id[j] - start;
  if (o < cnt) arr[j] = src[o];
}

__global__ void k_get_array(const float4* __restrict__ arr, const uint32_t* __restrict__ id,
                            float4* __restrict__ dst, uint32_t N) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < N) dst[id[j]] = arr[j];
}

// Host buffers the GPU can address (pinned, mapped): the records move
// between host memory and the state in one pass, in original order on the
// host side (coalesced over the host link), through the inverse of the
// stored order, inv[original index] = stored position.
__global__ void k_inverse(const uint32_t* __restrict__ id, uint32_t* __restrict__ inv, uint32_t N) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < N) inv[id[j]] = j;
}

__global__ void k_set_array_host(float4* __restrict__ arr, const uint32_t* __restrict__ inv,
                                 const float4* __restrict__ src, uint32_t start, uint32_t cnt) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o < cnt) arr[inv[start + o]] = src[o];
}

__global__ void k_get_array_host(const float4* __restrict__ arr, const uint32_t* __restrict__ inv,
                                 float4* __restrict__ dst, uint32_t N) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o < N) dst[o] = arr[inv[o]];
}

__global__ void k_sorted_hash(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff,
                              int S, uint32_t N, const float4* __restrict__ pos,
                              const uint32_t* __restrict__ id, uint2* __restrict__ out) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const int s = S == 1 ? 0 : scene_of(poff, S, j);
  const SceneDesc& d = sc[s];
  out[j] = make_uint2(cell_of(d.p, grid_pos(d.p, pos[j])), id[j] - d.p_off);
}

__global__ void k_cell_ranges(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ coff,
                              int S, uint32_t C, const uint32_t* __restrict__ start,
                              const uint32_t* __restrict__ count, uint32_t* __restrict__ cs,
                              uint32_t* __restrict__ ce) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const uint32_t po = sc[S == 1 ? 0 : scene_of(coff, S, c)].p_off;
  const uint32_t n = count[c];
  if (cs) cs[c] = n ? start[c] - po : kEmpty;
  if (ce) ce[c] = n ? start[c] + n - po : kEmpty;
}

// Per-scene kinetic energy, density sum, max |rho/rho0 - 1| and the count
// of non-finite coordinates.  Per-particle terms and the sum over a warp
// are FP32 (the GPU's FP64 rate is low); warp partials are summed in FP64.
__global__ void __launch_bounds__(kBlock) k_stats(const SceneDesc* __restrict__ sc,
                                                  const uint32_t* __restrict__ poff, int S,
                                                  uint32_t N, const float4* __restrict__ pos,
                                                  const float4* __restrict__ vel,
                                                  const float* __restrict__ dens,
                                                  double* __restrict__ acc) {
  int s = -1;
  float ke = 0.f, rho = 0.f, dev = 0.f, bad = 0.f;
  auto one = [&](uint32_t i, int sc_) {
    const SimParams& p = sc[sc_].p;
    const float4 x = pos[i], v = vel[i];
    float k = 0.5f * p.particleMass * (v.x * v.x + v.y * v.y + v.z * v.z);
    float r = dens ? dens[i] : 0.f;
    float dv = dens ? fabsf(r / p.restDensity - 1.f) : 0.f;
    bad += (float)(!isfinite(x.x) + !isfinite(x.y) + !isfinite(x.z) + !isfinite(v.x) +
                   !isfinite(v.y) + !isfinite(v.z));
    if (!(k == k) || isinf(k)) k = 0.f;
    if (!(r == r) || isinf(r)) r = 0.f;
    if (!(dv == dv) || isinf(dv)) dv = 0.f;
    ke += k;
    rho += r;
    dev = fmaxf(dev, dv);
  };
  if (S == 1) {  // grid-stride: each thread sums a few particles
    s = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) one(i, 0);
  } else {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) {
      s = scene_of(poff, S, i);
      one(i, s);
    }
  }
  auto warp_sum = [](float& a, float& b, float& c, float& d) {
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
      c = fmaxf(c, __shfl_xor_sync(0xffffffffu, c, o));
      d += __shfl_xor_sync(0xffffffffu, d, o);
    }
  };
  auto add = [&](int sc_, double a, double b, double c, double d) {
    atomicAdd(acc + 4 * sc_ + 0, a);
    atomicAdd(acc + 4 * sc_ + 1, b);
    atomicMax((unsigned long long*)(acc + 4 * sc_ + 2), (unsigned long long)__double_as_longlong(c));
    atomicAdd(acc + 4 * sc_ + 3, d);
  };
  // One scene in the whole block (always for a single scene): reduce over
  // the block (threads past N add zeros) and add once; otherwise per warp
  // where the warp is uniform, per thread where it is not.
  const uint32_t first = blockIdx.x * blockDim.x;
  const uint32_t last = min(first + blockDim.x, N) - 1;
  const int s_first = S == 1 ? 0 : scene_of(poff, S, first);
  if (S == 1 || s_first == scene_of(poff, S, last)) {
    warp_sum(ke, rho, dev, bad);
    __shared__ double part[kBlock / 32][4];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
      part[w][0] = ke;
      part[w][1] = rho;
      part[w][2] = dev;
      part[w][3] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = part[0][0], b = part[0][1], c = part[0][2], d = part[0][3];
      for (int k = 1; k < kBlock / 32; ++k) {
        a += part[k][0];
        b += part[k][1];
        c = fmax(c, part[k][2]);
        d += part[k][3];
      }
      add(s_first, a, b, c, d);
    }
    return;
  }
  const uint32_t peers = __match_any_sync(0xffffffffu, (uint32_t)s);
  if (peers == 0xffffffffu) {
    warp_sum(ke, rho, dev, bad);
    if ((threadIdx.x & 31) != 0) return;
  }
  if (s < 0) return;
  add(s, ke, rho, dev, bad);
}

// ---- persistent step ------------------------------------------------------
// K whole steps in one cooperative launch: every block runs every stage as a
// grid-stride loop over the same per-item device functions the separate
// kernels use, with a grid barrier between stages, so the results are those
// of enqueue_step bit for bit.  The launch is cooperative, so all blocks are
// resident; the barrier's waits are bounded: after kBarrierSpins polls a
// block sets bit 2 (kFlagBarrier) of `flags` and the barrier status, and
// every block leaves at its next barrier.
constexpr int kPThreads = 256;
constexpr int kPWarps = kPThreads / 32;
constexpr uint32_t kPTile = kPThreads * 8;            // scan tile
constexpr uint32_t kPBlockSortMax = kPWarps * kWarpSortMax;  // keys a block sorts in shared memory
constexpr uint32_t kBarrierSpins = 1u << 24;
constexpr uint32_t kFlagBarrier = 4u;

struct PersistArgs {
  const SceneDesc* sc;
  const uint32_t* poff;
  int S;
  uint32_t N, C;
  float4 *pos0, *pos1, *vel0, *vel1;
  uint32_t *id0, *id1;
  uint32_t *key, *rank, *slot, *dest, *count, *start, *tsum;
  float *dens, *pres;
  float2* dp;
  unsigned long long* masks;
  uint32_t* flags;
  uint32_t *sort_list, *sort_counters, *big_list, *sort_scratch;
  uint32_t* bar;  // [arrived, generation, status]
  uint32_t steps;
  int cp, cv;
  uint32_t spins;   // poll limit of a barrier wait (kBarrierSpins)
  uint32_t absent;  // a block that leaves at once (a test of the timeout), or ~0u
};

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Sense-reversing grid barrier: the last block to arrive resets the count
// and advances the generation; the others poll the generation (acquire).
__device__ bool grid_barrier(uint32_t* bar, uint32_t* flags, uint32_t max_spins) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t g = ld_acquire(bar + 1);
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      uint32_t spins = 0;
      while (ld_acquire(bar + 1) == g) {
        if (++spins > max_spins) {
          atomicOr(bar + 2, 1u);
          atomicOr(flags, kFlagBarrier);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *((volatile uint32_t*)(bar + 2)) == 0;
}

// Exclusive scan over the block of one value per thread; *total gets the sum.
__device__ __forceinline__ uint32_t p_block_scan(uint32_t v, uint32_t* wtot, uint32_t* total) {
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if ((int)lane >= o) x += y;
  }
  if (lane == 31) wtot[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < kPWarps ? wtot[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if ((int)lane >= o) t += y;
    }
    if (lane < kPWarps) wtot[lane] = t;  // inclusive warp offsets
  }
  __syncthreads();
  const uint32_t off = w ? wtot[w - 1] : 0u;
  *total = wtot[kPWarps - 1];
  __syncthreads();
  return off + x - v;
}

__global__ void __launch_bounds__(kPThreads, 4) k_persistent(PersistArgs a) {
  extern __shared__ uint32_t psm[];  // kPBlockSortMax words: a warp's or a block's cell ids
  __shared__ uint32_t wtot[32];
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nthr = gridDim.x * blockDim.x;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t gwarp = tid >> 5, nwarps = nthr >> 5;
  const uint32_t tiles = (a.C + kPTile - 1) / kPTile;
  float4* vel_v = a.cv ? a.vel1 : a.vel0;
  float4* vel_o = a.cv ? a.vel0 : a.vel1;
  int cp = a.cp;
  if (blockIdx.x == a.absent) return;
  for (uint32_t step = 0; step < a.steps; ++step) {
    float4 *pa = cp ? a.pos1 : a.pos0, *pb = cp ? a.pos0 : a.pos1;
    uint32_t *ia = cp ? a.id1 : a.id0, *ib = cp ? a.id0 : a.id1;
    // clear the cell counts and the sort lists
    for (uint32_t c = tid; c < a.C; c += nthr) a.count[c] = 0u;
    if (tid == 0) a.sort_counters[0] = a.sort_counters[1] = 0u;
    if (!grid_barrier(a.bar, a.flags, a.spins)) return;
    // integrate and count (whole warps over consecutive particles)
    for (uint32_t base = gwarp * 32; base < a.N; base += nwarps * 32)
      integrate_count_item(a.sc, a.poff, a.S, a.N, pa, vel_v, a.key, a.rank, a.count, a.flags, base + lane);
    if (!grid_barrier(a.bar, a.flags, a.spins)) return;
    // exclusive scan count -> start: tile sums, their scan (block 0), tiles
    for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x) {
      uint32_t sum = 0, tot;
      for (uint32_t k = 0; k < 8; ++k) {
        const uint32_t c = t * kPTile + threadIdx.x * 8 + k;
        if (c < a.C) sum += a.count[c];
      }
      p_block_scan(sum, wtot, &tot);
      if (threadIdx.x == 0) a.tsum[t] = tot;
    }
    if (!grid_barrier(a.bar, a.flags, a.spins)) return;
    if (blockIdx.x == 0) {
      uint32_t carry = 0;
      for (uint32_t t0 = 0; t0 < tiles; t0 += kPThreads) {
        const uint32_t t = t0 + threadIdx.x;
        const uint32_t v = t < tiles ? a.tsum[t] : 0u;
        uint32_t tot;
        const uint32_t e = p_block_scan(v, wtot, &tot);
        if (t < tiles) a.tsum[t] = carry + e;
        carry += tot;
      }
    }
    if (!grid_barrier(a.bar, a.flags, a.spins)) return;
    for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x) {
      uint32_t v[8], sum = 0, tot;
      for (uint32_t k = 0; k < 8; ++k) {
        const uint32_t c = t * kPTile + threadIdx.x * 8 + k;
        v[k] = c < a.C ? a.count[c] : 0u;
        sum += v[k];
      }
      uint32_t run = p_block_scan(sum, wtot, &tot) + a.tsum[t];
      for (uint32_t k = 0; k < 8; ++k) {
        const uint32_t c = t * kPTile + threadIdx.x * 8 + k;
        if (c < a.C) a.start[c] = run;
        run += v[k];
      }
    }
    if (!grid_barrier(a.bar, a.flags, a.spins)) return;
    // ids into their cells; cells that need their ids sorted
    for (uint32_t i = tid; i < a.N; i += nthr) a.slot[a.start[a.key[i]] + a.rank[i]] = ia[i];
    for (uint32_t base = gwarp * 32; base < a.C; base += nwarps * 32) {
      const uint32_t c = base + lane;
      const uint32_t n = c < a.C ? a.count[c] : 0u;
      const bool mid = n > kLinearRank && n <= kWarpSortMax, big = n > kWarpSortMax;
      const uint32_t bm = __ballot_sync(0xffffffffu, mid), bb = __ballot_sync(0xffffffffu, big);
      uint32_t base_m = 0, base_b = 0;
      if (lane == 0) {
        if (bm) base_m = atomicAdd(a.sort_counters + 0, (uint32_t)__popc(bm));
        if (bb) base_b = atomicAdd(a.sort_counters + 1, (uint32_t)__popc(bb));
      }
      base_m = __shfl_sync(0xffffffffu, base_m, 0);
      base_b = __shfl_sync(0xffffffffu, base_b, 0);
      const uint32_t below = (1u << lane) - 1u;
      if (mid) a.sort_list[base_m + (uint32_t)__popc(bm & below)] = c;
      if (big) a.big_list[base_b + (uint32_t)__popc(bb & below)] = c;
    }
    if (!grid_barrier(a.bar, a.flags, a.spins)) return;
    // sort: a warp per listed cell, then a block per big cell
    {
      const uint32_t nl = *((volatile uint32_t*)a.sort_counters);
      for (uint32_t q = gwarp; q < nl; q += nwarps) {
        const uint32_t c = a.sort_list[q];
        warp_sort_segment_smem(a.slot, a.start[c], a.count[c], lane, a.dest,
                               psm + (threadIdx.x >> 5) * kWarpSortMax);
      }
      __syncthreads();
      const uint32_t nb = *((volatile uint32_t*)(a.sort_counters + 1));
      for (uint32_t q = blockIdx.x; q < nb; q += gridDim.x) {
        const uint32_t c = a.big_list[q], n = a.count[c], s0 = a.start[c], m = pow2_at_least(n);
        uint32_t* bb = m <= kPBlockSortMax ? psm : a.sort_scratch + 2 * (size_t)s0;
        for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) bb[k] = k < n ? a.slot[s0 + k] : 0xffffffffu;
        __syncthreads();
        if (m <= kPBlockSortMax)
          bitonic(bb, m, threadIdx.x, blockDim.x, [] { __syncthreads(); });
        else
          bitonic(bb, m, threadIdx.x, blockDim.x, [] {
            __threadfence_block();
            __syncthreads();
          });
        for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) a.dest[bb[k]] = s0 + k;
        __syncthreads();
      }
    }
    if (!grid_barrier(a.bar, a.flags, a.spins)) return;
    for (uint32_t i = tid; i < a.N; i += nthr)
      place_item(a.sc, a.poff, a.S, a.N, pa, vel_v, ia, a.key, a.start, a.count, a.slot, a.dest, pb, vel_o,
                 ib, nullptr, i);
    if (!grid_barrier(a.bar, a.flags, a.spins)) return;
    for (uint32_t i = tid; i < a.N; i += nthr)
      density_item<true, false>(a.sc, a.poff, a.S, a.N, pb, a.start, a.count, a.dens, a.pres, a.dp, a.masks,
                         a.flags, i);
    if (!grid_barrier(a.bar, a.flags, a.spins)) return;
    const FeatOut no_feat = {nullptr, nullptr, nullptr};
    for (uint32_t i = tid; i < a.N; i += nthr)
      force_item<true, false, false>(a.sc, a.poff, a.S, a.N, pb, vel_o, a.dens, a.dp, a.start, a.count,
                              a.masks, vel_v, no_feat, i);
    if (!grid_barrier(a.bar, a.flags, a.spins)) return;
    cp = 1 - cp;
  }
}

}  // namespace
}  // namespace sph

using namespace sph;

struct SphSystem {
  int S = 0;
  uint32_t N = 0, C = 0;
  std::vector<SimParams> params;
  std::vector<uint32_t> poff, coff;  // S + 1 entries each
  SceneDesc* d_scenes = nullptr;
  uint32_t* d_poff = nullptr;
  uint32_t* d_coff = nullptr;
  float4* pos[2] = {nullptr, nullptr};
  float4* vel[2] = {nullptr, nullptr};
  uint32_t* id[2] = {nullptr, nullptr};
  uint32_t *key = nullptr, *rank = nullptr, *slot = nullptr;
  uint32_t* dest = nullptr;  // sorted position of each id of a crowded cell
  uint32_t *big_list = nullptr, *sort_scratch = nullptr;
  uint32_t *sort_list = nullptr, *sort_counters = nullptr;  // counters: list, big_list sizes
  unsigned big_blocks = 1, sort_blocks = 1;
  int sms = 1;                       // multiprocessors of the device
  uint32_t *count = nullptr, *start = nullptr, *scan_tmp = nullptr;
  float *dens = nullptr, *pres = nullptr;
  float2* dp = nullptr;               // per particle: 1/density, pressure (force pass)
  unsigned long long* masks = nullptr;  // kRows x N neighbour masks (null: walks without)
  uint32_t* flags = nullptr;
  double* stats = nullptr;
  float4* staging = nullptr;
  uint32_t* inv = nullptr;           // stored position of each original index (host transfers)
  bool inv_ok = false;               // inv matches the current order (cleared by every step)
  int cp = 0;  // pos/id buffer holding the state
  int cv = 0;  // vel buffer holding the state
  bool stepped = false;
  cudaStream_t stream = nullptr;
  bool own_stream = false;  // created here (destroyed here) or borrowed
  cudaStream_t cap_stream = nullptr;
  // the sort of the largest cells runs beside the warp sorts: a side stream
  // forked from and joined back into the step's stream by two events
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // graph_steps steps, keyed by cp at launch
  uint32_t graph_steps = 2;                         // steps per captured graph (even)
  int walk_shape = kDefaultShape;                   // index into kShapes
  // learned corrector
  SceneDesc* d_coarse = nullptr;     // scene table with timeStep * coarse_sub
  uint32_t coarse_sub = 0;
  void* mlp_img = nullptr;           // packed BF16 weights
  float* mlp_aux = nullptr;          // feature mean[16], inv_std[16], out_scale[3]
  bool model_set = false;
  float drift = -1.f;                // drift correction factor; < 0: (n-1)/(2n)
  float jerk = 0.f;                  // jerk correction factor; < 0: (n-1)/(2n)
  float4* vstart = nullptr;          // pre-integrate velocity of the coarse step (sorted)
  float4* hist = nullptr;            // per original index: previous dv_pre - dv_post
  bool hist_valid = false;
  uint16_t* feat = nullptr;          // N x 16 standardised features (BF16)
  float* mlp_y = nullptr;            // N x 3 corrections
  float4* bk_vel = nullptr;          // velocity checkpoint for the fallback
  double* stats_host = nullptr;      // pinned, 4 per scene
  cudaGraphExec_t lgraph[2] = {nullptr, nullptr};  // one learned coarse step, by cp parity
  uint64_t lgraph_key = 0;           // substeps and drift factor the learned graphs hold
  bool persistent = false;           // steps as one cooperative launch (k_persistent)
  unsigned persist_grid = 0;
  uint32_t* ptsum = nullptr;         // scan tile sums of the persistent step
  uint32_t* pbar = nullptr;          // its grid barrier: arrived, generation, status
  float4* clr_out = nullptr;         // caller's colour buffer (original order) or null
  float* dye_out = nullptr;          // caller's dye buffer (original order) or null
  std::vector<double> lr_ref[2];     // mean densities of the last two accepted steps
  int lr_refs = 0;                   // how many of lr_ref are valid for the current state
};

namespace {

int upload_scenes(SphSystem* s) {
  std::vector<SceneDesc> h(s->S);
  for (int i = 0; i < s->S; ++i) {
    h[i].p = s->params[i];
    h[i].p_off = s->poff[i];
    h[i].p_cnt = s->poff[i + 1] - s->poff[i];
    h[i].c_off = s->coff[i];
    h[i].c_cnt = s->coff[i + 1] - s->coff[i];
    h[i].inv_cell[0] = 1.f / h[i].p.cellSize.x;
    h[i].inv_cell[1] = 1.f / h[i].p.cellSize.y;
    h[i].inv_cell[2] = 1.f / h[i].p.cellSize.z;
  }
  SPH_CUDA(cudaMemcpyAsync(s->d_scenes, h.data(), sizeof(SceneDesc) * s->S, cudaMemcpyHostToDevice,
                           s->stream),
           "upload scene table");
  return cuda_check(cudaStreamSynchronize(s->stream), "upload scene table");
}

void drop_graphs(SphSystem* s) {
  for (auto& g : s->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  for (auto& g : s->lgraph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

inline uint32_t float_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, sizeof(u));
  return u;
}

// The stats kernel over the current state (into s->stats, cleared by the
// caller).  A single scene is reduced grid-stride by a few blocks per SM, so
// the FP64 atomics on the four totals stay few.
int launch_stats(SphSystem* s, cudaStream_t st) {
  const unsigned blocks = s->S == 1 ? std::min(grid_for(s->N, kBlock), 4u * (unsigned)s->sms)
                                    : grid_for(s->N, kBlock);
  k_stats<<<blocks, kBlock, 0, st>>>(s->d_scenes, s->d_poff, s->S, s->N, s->pos[s->cp], s->vel[s->cv],
                                     s->stepped ? s->dens : nullptr, s->stats);
  return cuda_check(cudaGetLastError(), "stats kernel");
}

// What one enqueued step uses besides the handle's buffers.
struct StepOpts {
  const SceneDesc* scenes = nullptr;  // scene table (fine or coarse time step)
  bool feat = false;                  // force pass also writes learned-corrector features
  FeatOut fo = {nullptr, nullptr, nullptr};
  float4* vel_start = nullptr;        // k_place also writes the pre-integrate velocity
};

template <bool kMask, int kThreads, int kMinBlocks, class Mark>
void launch_walks_shape(SphSystem* s, cudaStream_t st, int b, int v, const StepOpts& o, Mark& mark) {
  const unsigned g = grid_for(s->N, kThreads);
  k_density<kMask, kThreads, kMinBlocks><<<g, kThreads, 0, st>>>(
      o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->start, s->count, s->dens, s->pres, s->dp,
      s->masks, s->flags);
  mark();
  if (o.feat)
    k_force<kMask, kThreads, kMinBlocks, true><<<g, kThreads, 0, st>>>(
        o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->vel[1 - v], s->dens, s->dp, s->start,
        s->count, s->masks, s->vel[v], o.fo);
  else
    k_force<kMask, kThreads, kMinBlocks, false><<<g, kThreads, 0, st>>>(
        o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->vel[1 - v], s->dens, s->dp, s->start,
        s->count, s->masks, s->vel[v], o.fo);
}

inline size_t tile_smem_density(uint32_t slots) { return sizeof(TileTables) + 3 * sizeof(float) * slots; }
inline size_t tile_smem_force(uint32_t slots) { return sizeof(TileTables) + 2 * sizeof(float4) * slots; }
inline size_t tile_smem_pairs(uint32_t pairs) { return sizeof(TileTables) + (sizeof(float4) + sizeof(float2)) * pairs; }

template <int kThreads>
constexpr uint32_t pairs_cap() { return kThreads == 64 ? kPairs64 : (kThreads == 256 ? kPairs256 : kPairs128); }

template <int kThreads, class Mark>
void launch_density(SphSystem* s, cudaStream_t st, int b, const StepOpts& o, int kind, Mark& mark) {
  const unsigned g = grid_for(s->N, kThreads);
  constexpr int kMin = 1024 / kThreads;
  if (kind == 1 && kThreads == 128)
    k_density_tile<128><<<g, 128, tile_smem_density(kTileDensSlots), st>>>(
        o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->start, s->count, s->dens, s->pres, s->dp, s->masks,
        s->flags, kTileDensSlots);
  else if (kind == 2)
    k_density_pairs<kThreads, pairs_cap<kThreads>()><<<g, kThreads, tile_smem_pairs(pairs_cap<kThreads>()), st>>>(
        o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->start, s->count, s->dens, s->pres, s->dp, s->masks,
        s->flags);
  else
    k_density<true, kThreads, kMin><<<g, kThreads, 0, st>>>(o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->start,
                                                            s->count, s->dens, s->pres, s->dp, s->masks, s->flags);
  mark();
}

template <int kThreads>
void launch_force(SphSystem* s, cudaStream_t st, int b, int v, const StepOpts& o, int kind) {
  const unsigned g = grid_for(s->N, kThreads);
  constexpr int kMin = 1024 / kThreads;
  if (o.feat && kind == 2)  // the featured pass of the learned step: by cell fields
    k_force_fields<kThreads, kMin * 7 / 8, true><<<g, kThreads, 0, st>>>(
        o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->vel[1 - v], s->dp, s->start, s->masks, s->vel[v],
        s->dens, o.fo);
  else if (o.feat)  // the featured pass of the learned step: the global row walk
    k_force<true, 128, 8, true><<<grid_for(s->N, 128), 128, 0, st>>>(
        o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->vel[1 - v], s->dens, s->dp, s->start, s->count,
        s->masks, s->vel[v], o.fo);
  else if (kind == 1 && kThreads == 128)
    k_force_tile<128><<<g, 128, tile_smem_force(kTileForceSlots), st>>>(
        o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->vel[1 - v], s->dens, s->dp, s->start, s->count,
        s->masks, s->vel[v], kTileForceSlots);
  else if (kind == 2)
    k_force_fields<kThreads, kMin, false><<<g, kThreads, 0, st>>>(o.scenes, s->d_poff, s->S, s->N, s->pos[b],
                                                                  s->vel[1 - v], s->dp, s->start, s->masks,
                                                                  s->vel[v], nullptr, FeatOut{});
  else if (kind == 3 && kThreads <= 128)
    k_force_coop<kThreads <= 128 ? kThreads : 128><<<g, kThreads, 0, st>>>(
        o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->vel[1 - v], s->dp, s->start, s->masks, s->vel[v]);
  else
    k_force<true, kThreads, kMin, false><<<g, kThreads, 0, st>>>(
        o.scenes, s->d_poff, s->S, s->N, s->pos[b], s->vel[1 - v], s->dens, s->dp, s->start, s->count,
        s->masks, s->vel[v], o.fo);
}

template <bool kMask, class Mark>
void launch_walks(SphSystem* s, cudaStream_t st, int b, int v, const StepOpts& o, Mark& mark) {
  const WalkShape& w = kShapes[s->walk_shape];
  if (kMask) {
    switch (w.threads) {
      case 64:
        launch_density<64>(s, st, b, o, w.dens, mark);
        launch_force<64>(s, st, b, v, o, w.force);
        break;
      case 256:
        launch_density<256>(s, st, b, o, w.dens, mark);
        launch_force<256>(s, st, b, v, o, w.force);
        break;
      default:
        launch_density<128>(s, st, b, o, w.dens, mark);
        launch_force<128>(s, st, b, v, o, w.force);
        break;
    }
    return;
  }
  switch (w.threads) {
    case 64: launch_walks_shape<false, 64, 16>(s, st, b, v, o, mark); break;
    case 256: launch_walks_shape<false, 256, 4>(s, st, b, v, o, mark); break;
    default: launch_walks_shape<false, 128, 8>(s, st, b, v, o, mark); break;
  }
}

// Shared memory the staged walks may use (set once per handle).
int tile_attributes() {
  SPH_CUDA(cudaFuncSetAttribute(k_density_tile<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tile_smem_density(kTileDensSlots)), "staged density walk shared memory");
  SPH_CUDA(cudaFuncSetAttribute(k_force_tile<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tile_smem_force(kTileForceSlots)), "staged force walk shared memory");
  SPH_CUDA(cudaFuncSetAttribute(k_density_pairs<64, kPairs64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tile_smem_pairs(kPairs64)), "staged density walk shared memory");
  SPH_CUDA(cudaFuncSetAttribute(k_density_pairs<128, kPairs128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tile_smem_pairs(kPairs128)), "staged density walk shared memory");
  SPH_CUDA(cudaFuncSetAttribute(k_density_pairs<256, kPairs256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tile_smem_pairs(kPairs256)), "staged density walk shared memory");
  return SPH_OK;
}

// Enqueues one step on `st`, advancing s->cp.  With `ev` (kStepStages + 1
// events) an event is recorded before the first stage and after each one.
constexpr int kStepStages = 6;
int enqueue_step(SphSystem* s, cudaStream_t st, cudaEvent_t* ev = nullptr,
                 const StepOpts* opts = nullptr) {
  StepOpts o;
  if (opts) o = *opts;
  if (!o.scenes) o.scenes = s->d_scenes;
  const SceneDesc* sc = o.scenes;
  const unsigned gN = grid_for(s->N, kBlock);
  const int a = s->cp, b = 1 - s->cp, v = s->cv;
  int e = 0;
  auto mark = [&]() {
    if (ev) cudaEventRecord(ev[e++], st);
  };
  mark();
  SPH_CUDA(cudaMemsetAsync(s->count, 0, sizeof(uint32_t) * s->C, st), "step: clear counts");
  k_integrate_count<<<gN, kBlock, 0, st>>>(sc, s->d_poff, s->S, s->N, s->pos[a], s->vel[v],
                                           s->key, s->rank, s->count, s->flags);
  mark();
  // the scan also lists the cells whose id segments need sorting (more than
  // kLinearRank particles: up to kWarpSortMax into sort_list, the rest into
  // big_list)
  SPH_TRY(exclusive_scan_lists(s->count, s->start, s->C, s->scan_tmp,
                               ScanLists{kLinearRank, kWarpSortMax, s->sort_list, s->big_list, s->sort_counters},
                               st));
  mark();
  k_scatter_ids<<<gN, kBlock, 0, st>>>(s->N, s->key, s->rank, s->id[a], s->start, s->slot);
  // the few cells above kWarpSortMax (a block each) beside the warp sorts:
  // the two kernels sort disjoint cells
  SPH_CUDA(cudaEventRecord(s->fork_ev, st), "step: fork");
  SPH_CUDA(cudaStreamWaitEvent(s->side, s->fork_ev, 0), "step: fork");
  k_rank_big_cells<<<s->big_blocks, kBigThreads, kBigRankSmem, s->side>>>(
      s->start, s->count, s->slot, s->big_list, s->sort_counters + 1, s->sort_scratch, s->dest);
  SPH_CUDA(cudaEventRecord(s->join_ev, s->side), "step: join");
  // cells of up to kWarpSortMax ids: ranked by buckets (k_rank_cells; the
  // few whose ids bunch into one bucket are sorted by the same block)
  k_rank_cells<<<s->sort_blocks, kRankThreads, 0, st>>>(s->start, s->count, s->slot, s->sort_list,
                                                        s->sort_counters, s->dest);
  SPH_CUDA(cudaStreamWaitEvent(st, s->join_ev, 0), "step: join");
  mark();
  k_place<<<gN, kBlock, 0, st>>>(sc, s->d_poff, s->S, s->N, s->pos[a], s->vel[v], s->id[a],
                                 s->key, s->start, s->count, s->slot, s->dest, s->pos[b], s->vel[1 - v],
                                 s->id[b], o.vel_start);
  mark();
  if (s->masks)
    launch_walks<true>(s, st, b, v, o, mark);
  else
    launch_walks<false>(s, st, b, v, o, mark);
  if (s->clr_out)
    k_color<<<gN, kBlock, 0, st>>>(sc, s->d_poff, s->S, s->N, s->pos[b], s->vel[1 - v], s->vel[v],
                                   s->dens, s->start, s->count, s->id[b], s->clr_out, s->dye_out);
  mark();
  SPH_CUDA(cudaGetLastError(), "step kernels");
  s->cp = b;
  s->stepped = true;
  s->inv_ok = false;
  return SPH_OK;
}

int build_graph(SphSystem* s) {
  const int cp0 = s->cp;
  if (!s->cap_stream)
    SPH_CUDA(cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking), "capture stream");
  SPH_CUDA(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  int rc = SPH_OK;
  for (uint32_t k = 0; k < s->graph_steps && rc == SPH_OK; ++k) rc = enqueue_step(s, s->cap_stream);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s->cap_stream, &g);
  s->cp = cp0;
  if (rc != SPH_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  SPH_CUDA(e, "end capture");
  const cudaError_t ie = cudaGraphInstantiate(&s->graph[cp0], g, 0);
  cudaGraphDestroy(g);
  return cuda_check(ie, "instantiate step graph");
}

void free_all(SphSystem* s) {
  drop_graphs(s);
  void* bufs[] = {s->d_scenes, s->d_poff, s->d_coff, s->pos[0], s->pos[1], s->vel[0], s->vel[1],
                  s->id[0], s->id[1], s->key, s->rank, s->slot, s->dest, s->count, s->start, s->scan_tmp,
                  s->dens, s->pres, s->dp, s->masks, s->flags, s->stats, s->staging, s->inv, s->d_coarse,
                  s->mlp_img, s->mlp_aux, s->feat, s->mlp_y, s->bk_vel, s->vstart, s->hist, s->ptsum, s->pbar,
                  s->big_list, s->sort_counters, s->sort_list, s->sort_scratch};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
  if (s->side) cudaStreamDestroy(s->side);
  if (s->fork_ev) cudaEventDestroy(s->fork_ev);
  if (s->join_ev) cudaEventDestroy(s->join_ev);
  if (s->stats_host) cudaFreeHost(s->stats_host);
}

template <class T>
int dalloc(T** p, size_t n, const char* what) {
  return cuda_check(cudaMalloc((void**)p, sizeof(T) * (n ? n : 1)), what);
}

int create(const SimParams* scenes, uint32_t count, SphSystem** out) {
  if (!scenes || !out || count == 0) return fail(SPH_ERR_ARG, "sph_create: bad arguments");
  *out = nullptr;
  uint64_t n = 0, c = 0;
  for (uint32_t i = 0; i < count; ++i) {
    SPH_TRY(validate_params(scenes[i], true));
    if (scenes[i].numParticles == 0) return fail(SPH_ERR_PARAMS, "scene %u has no particles", i);
    n += scenes[i].numParticles;
    c += scenes[i].numCells;
  }
  if (n >= (1ull << 31) || c >= (1ull << 31))
    return fail(SPH_ERR_PARAMS, "%llu particles / %llu cells exceed one handle", (unsigned long long)n,
                (unsigned long long)c);
  SphSystem* s = new SphSystem();
  s->S = (int)count;
  s->N = (uint32_t)n;
  s->C = (uint32_t)c;
  s->params.assign(scenes, scenes + count);
  s->poff.resize(count + 1);
  s->coff.resize(count + 1);
  s->poff[0] = s->coff[0] = 0;
  for (uint32_t i = 0; i < count; ++i) {
    s->poff[i + 1] = s->poff[i] + scenes[i].numParticles;
    s->coff[i + 1] = s->coff[i] + scenes[i].numCells;
  }
  int rc = SPH_OK;
#define ALLOC(ptr, n, what) \
  if (rc == SPH_OK) rc = dalloc(&(ptr), (n), (what))
  ALLOC(s->d_scenes, count, "scene table");
  ALLOC(s->d_poff, count + 1, "scene offsets");
  ALLOC(s->d_coff, count + 1, "cell offsets");
  for (int k = 0; k < 2; ++k) {
    ALLOC(s->pos[k], n, "positions");
    ALLOC(s->vel[k], n, "velocities");
    ALLOC(s->id[k], n, "particle ids");
  }
  ALLOC(s->key, n, "cell keys");
  ALLOC(s->rank, n, "cell ranks");
  ALLOC(s->slot, n, "cell slots");
  ALLOC(s->dest, n, "sorted positions");
  ALLOC(s->big_list, n / (kWarpSortMax + 1) + 1, "crowded-cell list");
  ALLOC(s->sort_list, n / (kLinearRank + 1) + 1, "cell sort list");
  ALLOC(s->sort_counters, 2, "cell sort list sizes");
  ALLOC(s->sort_scratch, 2 * n, "cell sort scratch");
  ALLOC(s->count, c, "cell counts");
  ALLOC(s->start, c, "cell starts");
  ALLOC(s->scan_tmp, scan_scratch_words(c), "scan scratch");
  ALLOC(s->dens, n, "density");
  ALLOC(s->dp, n, "inverse density and pressure");
  ALLOC(s->pres, n, "pressure");
  ALLOC(s->flags, 1, "flags");
  bool use_masks = SPH_WALK_MASKS != 0;
  for (uint32_t i = 0; i < count; ++i) use_masks &= scenes[i].maxParInCell <= kMaskMaxPerCell;
  if (use_masks) ALLOC(s->masks, (size_t)kRows * n, "neighbour masks");
  ALLOC(s->stats, 4 * (size_t)count, "stats");
#undef ALLOC
  if (rc == SPH_OK) rc = cuda_check(cudaStreamCreate(&s->stream), "stream");
  s->own_stream = rc == SPH_OK;
  if (rc == SPH_OK) rc = cuda_check(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking), "side stream");
  if (rc == SPH_OK) rc = cuda_check(cudaEventCreateWithFlags(&s->fork_ev, cudaEventDisableTiming), "fork event");
  if (rc == SPH_OK) rc = cuda_check(cudaEventCreateWithFlags(&s->join_ev, cudaEventDisableTiming), "join event");
  if (rc == SPH_OK)
    rc = cuda_check(cudaFuncSetAttribute(k_rank_big_cells, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kBigRankSmem),
                    "crowded-cell ranking shared memory");
  if (rc == SPH_OK) rc = tile_attributes();
  if (rc == SPH_OK) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    s->big_blocks = (unsigned)(sms > 0 ? sms : 1);
    s->sms = sms > 0 ? sms : 1;
    s->sort_blocks = (unsigned)(sms > 0 ? 8 * sms : 8);
  }
  if (rc == SPH_OK) {
    for (int k = 0; k < 2; ++k) {
      cudaMemsetAsync(s->pos[k], 0, sizeof(float4) * n, s->stream);
      cudaMemsetAsync(s->vel[k], 0, sizeof(float4) * n, s->stream);
    }
    cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), s->stream);
    cudaMemsetAsync(s->dens, 0, sizeof(float) * n, s->stream);
    cudaMemsetAsync(s->pres, 0, sizeof(float) * n, s->stream);
    cudaMemsetAsync(s->scan_tmp, 0, sizeof(uint32_t), s->stream);  // the scan's ticket counter
    k_iota<<<grid_for(n, kBlock), kBlock, 0, s->stream>>>(s->id[0], (uint32_t)n);
    rc = cuda_check(cudaGetLastError(), "init");
  }
  if (rc == SPH_OK)
    rc = cuda_check(cudaMemcpyAsync(s->d_poff, s->poff.data(), sizeof(uint32_t) * (count + 1),
                                    cudaMemcpyHostToDevice, s->stream),
                    "offsets");
  if (rc == SPH_OK)
    rc = cuda_check(cudaMemcpyAsync(s->d_coff, s->coff.data(), sizeof(uint32_t) * (count + 1),
                                    cudaMemcpyHostToDevice, s->stream),
                    "offsets");
  if (rc == SPH_OK) rc = upload_scenes(s);
  if (rc != SPH_OK) {
    free_all(s);
    if (s->stream && s->own_stream) cudaStreamDestroy(s->stream);
    delete s;
    return rc;
  }
  *out = s;
  return SPH_OK;
}

int ensure_staging(SphSystem* s) {
  if (!s->staging) return dalloc(&s->staging, s->N, "staging buffer");
  return SPH_OK;
}

// The device address of a host buffer the GPU can reach (pinned and mapped
// into the address space), or null for pageable memory.
const void* device_view(const void* host) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// inv from the stored order of the current state.
int refresh_inverse(SphSystem* s) {
  if (s->inv_ok) return SPH_OK;
  if (!s->inv) SPH_TRY(dalloc(&s->inv, s->N, "inverse order"));
  k_inverse<<<grid_for(s->N, kBlock), kBlock, 0, s->stream>>>(s->id[s->cp], s->inv, s->N);
  SPH_CUDA(cudaGetLastError(), "inverse order");
  s->inv_ok = true;
  return SPH_OK;
}

}  // namespace

extern "C" {

int sph_create(const SimParams* params, SphSystem** out) { return create(params, 1, out); }

int sph_create_ensemble(const SimParams* scenes, uint32_t count, SphSystem** out) {
  return create(scenes, count, out);
}

int sph_destroy(SphSystem* s) {
  if (!s) return SPH_OK;
  cudaStreamSynchronize(s->stream);
  free_all(s);
  if (s->own_stream) cudaStreamDestroy(s->stream);
  delete s;
  return SPH_OK;
}

int sph_set_stream(SphSystem* s, void* stream) {
  if (!s) return fail(SPH_ERR_ARG, "null handle");
  SPH_CUDA(cudaStreamSynchronize(s->stream), "set_stream: drain");
  if (s->own_stream) cudaStreamDestroy(s->stream);
  s->stream = nullptr;
  s->own_stream = false;
  if (stream) {
    s->stream = (cudaStream_t)stream;  // borrowed: never destroyed here
  } else {
    SPH_CUDA(cudaStreamCreate(&s->stream), "stream");
    s->own_stream = true;
  }
  return SPH_OK;
}

int sph_set_params(SphSystem* s, uint32_t scene, const SimParams* p) {
  if (!s || !p || scene >= (uint32_t)s->S) return fail(SPH_ERR_ARG, "set_params: bad arguments");
  s->lr_refs = 0;  // the learned step's density history no longer applies
  const SimParams& o = s->params[scene];
  if (p->numParticles != o.numParticles || p->numCells != o.numCells ||
      p->gridSize.x != o.gridSize.x || p->gridSize.y != o.gridSize.y || p->gridSize.z != o.gridSize.z)
    return fail(SPH_ERR_PARAMS, "set_params: particle count and grid cannot change");
  SPH_TRY(validate_params(*p, true));
  s->params[scene] = *p;
  s->coarse_sub = 0;  // the learned step's coarse table is rebuilt from the new parameters
  return upload_scenes(s);
}

int sph_get_params(SphSystem* s, uint32_t scene, SimParams* out) {
  if (!s || !out || scene >= (uint32_t)s->S) return fail(SPH_ERR_ARG, "get_params: bad arguments");
  *out = s->params[scene];
  return SPH_OK;
}

uint32_t sph_num_scenes(const SphSystem* s) { return s ? (uint32_t)s->S : 0; }
uint32_t sph_num_particles(const SphSystem* s) { return s ? s->N : 0; }
uint32_t sph_num_cells(const SphSystem* s) { return s ? s->C : 0; }
uint32_t sph_scene_offset(const SphSystem* s, uint32_t scene) {
  return (s && scene <= (uint32_t)s->S) ? s->poff[scene] : 0;
}

int sph_set_array(SphSystem* s, uint32_t which, const sph_float4* data, uint32_t start,
                  uint32_t count, int src_on_device) {
  if (!s || !data || which > SPH_ARRAY_VEL) return fail(SPH_ERR_ARG, "set_array: bad arguments");
  s->lr_refs = 0;  // the learned step's density history no longer applies
  if ((uint64_t)start + count > s->N) return fail(SPH_ERR_ARG, "set_array: range beyond %u particles", s->N);
  if (count == 0) return SPH_OK;
  if (!src_on_device) {
    if (const void* dv = device_view(data)) {  // pinned: one pass over the host link
      SPH_TRY(refresh_inverse(s));
      float4* arr = which == SPH_ARRAY_POS ? s->pos[s->cp] : s->vel[s->cv];
      k_set_array_host<<<grid_for(count, kBlock), kBlock, 0, s->stream>>>(arr, s->inv, (const float4*)dv,
                                                                          start, count);
      SPH_CUDA(cudaGetLastError(), "set_array kernel");
      return cuda_check(cudaStreamSynchronize(s->stream), "set_array sync");
    }
  }
  SPH_TRY(ensure_staging(s));
  SPH_CUDA(cudaMemcpyAsync(s->staging, data, sizeof(float4) * count,
                           src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s->stream),
           "set_array copy");
  float4* arr = which == SPH_ARRAY_POS ? s->pos[s->cp] : s->vel[s->cv];
  k_set_array<<<grid_for(s->N, kBlock), kBlock, 0, s->stream>>>(arr, s->id[s->cp], s->staging, start,
                                                                count, s->N);
  SPH_CUDA(cudaGetLastError(), "set_array kernel");
  if (!src_on_device) SPH_CUDA(cudaStreamSynchronize(s->stream), "set_array sync");
  return SPH_OK;
}

int sph_get_array(SphSystem* s, uint32_t which, sph_float4* out, int dst_on_device) {
  if (!s || !out || which > SPH_ARRAY_VEL) return fail(SPH_ERR_ARG, "get_array: bad arguments");
  const float4* arr = which == SPH_ARRAY_POS ? s->pos[s->cp] : s->vel[s->cv];
  float4* dst = (float4*)out;
  if (!dst_on_device) {
    if (const void* dv = device_view(out)) {  // pinned: one pass over the host link
      SPH_TRY(refresh_inverse(s));
      k_get_array_host<<<grid_for(s->N, kBlock), kBlock, 0, s->stream>>>(arr, s->inv, (float4*)dv, s->N);
      SPH_CUDA(cudaGetLastError(), "get_array kernel");
      return cuda_check(cudaStreamSynchronize(s->stream), "get_array sync");
    }
    SPH_TRY(ensure_staging(s));
    dst = s->staging;
  }
  k_get_array<<<grid_for(s->N, kBlock), kBlock, 0, s->stream>>>(arr, s->id[s->cp], dst, s->N);
  SPH_CUDA(cudaGetLastError(), "get_array kernel");
  if (!dst_on_device) {
    SPH_CUDA(cudaMemcpyAsync(out, s->staging, sizeof(float4) * s->N, cudaMemcpyDeviceToHost, s->stream),
             "get_array copy");
    SPH_CUDA(cudaStreamSynchronize(s->stream), "get_array sync");
  }
  return SPH_OK;
}

static int persistent_steps(SphSystem* s, uint32_t steps, uint32_t spins = kBarrierSpins,
                            uint32_t absent = ~0u) {
  PersistArgs a;
  a.spins = spins;
  a.absent = absent;
  a.sc = s->d_scenes;
  a.poff = s->d_poff;
  a.S = s->S;
  a.N = s->N;
  a.C = s->C;
  a.pos0 = s->pos[0];
  a.pos1 = s->pos[1];
  a.vel0 = s->vel[0];
  a.vel1 = s->vel[1];
  a.id0 = s->id[0];
  a.id1 = s->id[1];
  a.key = s->key;
  a.rank = s->rank;
  a.slot = s->slot;
  a.dest = s->dest;
  a.count = s->count;
  a.start = s->start;
  a.tsum = s->ptsum;
  a.dens = s->dens;
  a.pres = s->pres;
  a.dp = s->dp;
  a.masks = s->masks;
  a.flags = s->flags;
  a.sort_list = s->sort_list;
  a.sort_counters = s->sort_counters;
  a.big_list = s->big_list;
  a.sort_scratch = s->sort_scratch;
  a.bar = s->pbar;
  a.steps = steps;
  a.cp = s->cp;
  a.cv = s->cv;
  SPH_CUDA(cudaMemsetAsync(s->pbar, 0, 3 * sizeof(uint32_t), s->stream), "persistent: barrier");
  void* args[] = {&a};
  SPH_CUDA(cudaLaunchCooperativeKernel((const void*)k_persistent, dim3(s->persist_grid), dim3(kPThreads),
                                       args, kPWarps * kWarpSortMax * sizeof(uint32_t), s->stream),
           "persistent step launch");
  if (steps & 1) s->cp = 1 - s->cp;
  return SPH_OK;
}

int sph_persistent_withheld(SphSystem* s, uint32_t* flags) {
  if (!s || !flags) return fail(SPH_ERR_ARG, "persistent_withheld: bad arguments");
  if (!s->persistent || !s->persist_grid) return fail(SPH_ERR_ARG, "persistent_withheld: persistent stepping is off");
  const int cp = s->cp;
  SPH_TRY(persistent_steps(s, 1, 4096u, 0u));
  s->cp = cp;  // the step did not happen
  return sph_flags(s, flags);
}

int sph_set_persistent(SphSystem* s, int on) {
  if (!s) return fail(SPH_ERR_ARG, "null handle");
  if (!on) {
    s->persistent = false;
    return SPH_OK;
  }
  if (!s->masks) return fail(SPH_ERR_UNSUPPORTED, "set_persistent: needs the neighbour masks (maxParInCell <= 21)");
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  SPH_CUDA(cudaGetDevice(&dev), "set_persistent");
  SPH_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev), "set_persistent");
  if (!coop) return fail(SPH_ERR_UNSUPPORTED, "set_persistent: no cooperative launch on this device");
  SPH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "set_persistent");
  SPH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persistent, kPThreads,
                                                         kPWarps * kWarpSortMax * sizeof(uint32_t)),
           "set_persistent: occupancy");
  if (per_sm < 1) return fail(SPH_ERR_UNSUPPORTED, "set_persistent: kernel does not fit an SM");
  if (!s->ptsum) SPH_TRY(dalloc(&s->ptsum, (s->C + kPTile - 1) / kPTile + 1, "persistent tile sums"));
  if (!s->pbar) SPH_TRY(dalloc(&s->pbar, 3, "persistent barrier"));
  s->persist_grid = (unsigned)(per_sm * sms);
  s->persistent = true;
  return SPH_OK;
}

int sph_step(SphSystem* s, uint32_t steps) {
  if (!s) return fail(SPH_ERR_ARG, "null handle");
  s->lr_refs = 0;  // the learned step's density history no longer applies
  if (s->persistent && !s->clr_out) {
    if (steps) {
      SPH_TRY(persistent_steps(s, steps));
      s->stepped = true;
      s->inv_ok = false;
    }
    return SPH_OK;
  }
  uint32_t done = 0;
  const uint32_t gs = s->graph_steps;
  if (steps >= gs) {
    if (!s->graph[s->cp]) SPH_TRY(build_graph(s));
    for (; done + gs <= steps; done += gs)
      SPH_CUDA(cudaGraphLaunch(s->graph[s->cp], s->stream), "step graph launch");
  }
  for (; done < steps; ++done) SPH_TRY(enqueue_step(s, s->stream));
  if (steps) {
    s->stepped = true;
    s->inv_ok = false;
  }
  return SPH_OK;
}

int sph_set_graph_steps(SphSystem* s, uint32_t steps_per_graph) {
  if (!s || steps_per_graph < 2 || steps_per_graph % 2)
    return fail(SPH_ERR_ARG, "set_graph_steps: need an even count >= 2");
  SPH_CUDA(cudaStreamSynchronize(s->stream), "set_graph_steps: drain");
  drop_graphs(s);
  s->graph_steps = steps_per_graph;
  return SPH_OK;
}

int sph_set_color_output(SphSystem* s, sph_float4* clr, float* dye) {
  if (!s) return fail(SPH_ERR_ARG, "null handle");
  if (!clr && dye) return fail(SPH_ERR_ARG, "set_color_output: dye needs a colour buffer");
  s->clr_out = (float4*)clr;
  s->dye_out = dye;
  drop_graphs(s);  // the step graphs hold the old pointers
  return SPH_OK;
}

int sph_set_walk_shape(SphSystem* s, uint32_t shape) {
  if (!s || shape >= (uint32_t)kWalkShapes) return fail(SPH_ERR_ARG, "set_walk_shape: bad shape");
  SPH_CUDA(cudaStreamSynchronize(s->stream), "set_walk_shape: drain");
  drop_graphs(s);
  s->walk_shape = (int)shape;
  return SPH_OK;
}

int sph_get_walk_shape(SphSystem* s, uint32_t* shape, uint32_t* threads) {
  if (!s) return fail(SPH_ERR_ARG, "null handle");
  if (shape) *shape = (uint32_t)s->walk_shape;
  if (threads) *threads = (uint32_t)kShapes[s->walk_shape].threads;
  return SPH_OK;
}

int sph_autotune(SphSystem* s, uint32_t trial_steps, float* ms_per_step, uint32_t* chosen) {
  if (!s || trial_steps == 0) return fail(SPH_ERR_ARG, "autotune: bad arguments");
  s->lr_refs = 0;  // the learned step's density history no longer applies
  SPH_CUDA(cudaStreamSynchronize(s->stream), "autotune: drain");
  // Save the state so that tuning leaves the simulation where it was.
  float4 *sp = nullptr, *sv = nullptr;
  uint32_t* si = nullptr;
  int rc = dalloc(&sp, s->N, "autotune: saved positions");
  if (rc == SPH_OK) rc = dalloc(&sv, s->N, "autotune: saved velocities");
  if (rc == SPH_OK) rc = dalloc(&si, s->N, "autotune: saved ids");
  const int cp0 = s->cp, cv0 = s->cv, shape0 = s->walk_shape;
  const bool stepped0 = s->stepped;
  if (rc == SPH_OK) {
    cudaMemcpyAsync(sp, s->pos[cp0], sizeof(float4) * s->N, cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(sv, s->vel[cv0], sizeof(float4) * s->N, cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(si, s->id[cp0], sizeof(uint32_t) * s->N, cudaMemcpyDeviceToDevice, s->stream);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (rc == SPH_OK) rc = cuda_check(cudaEventCreate(&e0), "autotune: event");
  if (rc == SPH_OK) rc = cuda_check(cudaEventCreate(&e1), "autotune: event");
  float best = 0.f;
  int best_shape = shape0;
  for (int k = 0; k < kWalkShapes && rc == SPH_OK; ++k) {
    s->walk_shape = k;
    rc = enqueue_step(s, s->stream);  // warm-up
    if (rc == SPH_OK) rc = cuda_check(cudaEventRecord(e0, s->stream), "autotune: record");
    for (uint32_t t = 0; t < trial_steps && rc == SPH_OK; ++t) rc = enqueue_step(s, s->stream);
    if (rc == SPH_OK) rc = cuda_check(cudaEventRecord(e1, s->stream), "autotune: record");
    if (rc == SPH_OK) rc = cuda_check(cudaEventSynchronize(e1), "autotune: sync");
    float ms = 0.f;
    if (rc == SPH_OK) rc = cuda_check(cudaEventElapsedTime(&ms, e0, e1), "autotune: elapsed");
    ms /= (float)trial_steps;
    if (ms_per_step) ms_per_step[k] = ms;
    if (rc == SPH_OK && (k == 0 || ms < best)) {
      best = ms;
      best_shape = k;
    }
    // restore the saved state for the next candidate
    if (rc == SPH_OK) {
      s->cp = cp0;
      s->cv = cv0;
      cudaMemcpyAsync(s->pos[cp0], sp, sizeof(float4) * s->N, cudaMemcpyDeviceToDevice, s->stream);
      cudaMemcpyAsync(s->vel[cv0], sv, sizeof(float4) * s->N, cudaMemcpyDeviceToDevice, s->stream);
      cudaMemcpyAsync(s->id[cp0], si, sizeof(uint32_t) * s->N, cudaMemcpyDeviceToDevice, s->stream);
    }
  }
  if (rc == SPH_OK) rc = cuda_check(cudaStreamSynchronize(s->stream), "autotune: restore");
  s->walk_shape = rc == SPH_OK ? best_shape : shape0;
  s->stepped = stepped0 || rc == SPH_OK;
  s->inv_ok = false;
  drop_graphs(s);
  if (chosen) *chosen = (uint32_t)s->walk_shape;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (sp) cudaFree(sp);
  if (sv) cudaFree(sv);
  if (si) cudaFree(si);
  return rc;
}

namespace {

// Scene table whose time step is `sub` times the scenes' own.
int ensure_coarse(SphSystem* s, uint32_t sub) {
  if (!s->d_coarse) SPH_TRY(dalloc(&s->d_coarse, s->S, "coarse scene table"));
  std::vector<SceneDesc> h(s->S);
  for (int i = 0; i < s->S; ++i) {
    h[i].p = s->params[i];
    h[i].p.timeStep = s->params[i].timeStep * (float)sub;
    h[i].p_off = s->poff[i];
    h[i].p_cnt = s->poff[i + 1] - s->poff[i];
    h[i].c_off = s->coff[i];
    h[i].c_cnt = s->coff[i + 1] - s->coff[i];
    h[i].inv_cell[0] = 1.f / h[i].p.cellSize.x;
    h[i].inv_cell[1] = 1.f / h[i].p.cellSize.y;
    h[i].inv_cell[2] = 1.f / h[i].p.cellSize.z;
  }
  SPH_CUDA(cudaMemcpyAsync(s->d_coarse, h.data(), sizeof(SceneDesc) * s->S, cudaMemcpyHostToDevice,
                           s->stream),
           "coarse scene table");
  SPH_CUDA(cudaStreamSynchronize(s->stream), "coarse scene table");
  s->coarse_sub = sub;
  return SPH_OK;
}

// Per-scene mean density of the last step and non-finite counts (host).
int scene_stats(SphSystem* s, std::vector<double>& out) {
  out.assign(4 * s->S, 0.0);
  return sph_stats(s, out.data());
}

}  // namespace

int sph_learned_set_model(SphSystem* s, const float* params, const float* feat_stats,
                          const float* out_scale) {
  if (!s || !params || !feat_stats || !out_scale) return fail(SPH_ERR_ARG, "set_model: null argument");
  const int np = sph_mlp_param_count();
  float* dprm = nullptr;
  SPH_TRY(dalloc(&dprm, np, "model parameters"));
  if (!s->mlp_img) SPH_TRY(dalloc((uint8_t**)&s->mlp_img, sph_mlp_packed_bytes(), "packed model"));
  if (!s->mlp_aux) SPH_TRY(dalloc(&s->mlp_aux, 35, "model statistics"));
  int rc = cuda_check(cudaMemcpyAsync(dprm, params, sizeof(float) * np, cudaMemcpyHostToDevice,
                                      s->stream), "model upload");
  if (rc == SPH_OK) rc = cuda_check(cudaMemcpyAsync(s->mlp_aux, feat_stats, sizeof(float) * 32,
                                                    cudaMemcpyHostToDevice, s->stream), "model upload");
  if (rc == SPH_OK) rc = cuda_check(cudaMemcpyAsync(s->mlp_aux + 32, out_scale, sizeof(float) * 3,
                                                    cudaMemcpyHostToDevice, s->stream), "model upload");
  if (rc == SPH_OK) rc = sph_mlp_pack(dprm, s->mlp_img, s->stream);
  if (rc == SPH_OK) rc = cuda_check(cudaStreamSynchronize(s->stream), "model upload");
  cudaFree(dprm);
  s->model_set = rc == SPH_OK;
  return rc;
}

int sph_learned_set_options(SphSystem* s, float drift, float jerk) {
  if (!s || !(drift == drift) || !(jerk == jerk))
    return fail(SPH_ERR_ARG, "learned_set_options: bad arguments");
  s->drift = drift;
  s->jerk = jerk;
  return SPH_OK;
}

int sph_features_step(SphSystem* s, uint32_t substeps, float* feat_raw, uint32_t* ids) {
  if (!s || substeps == 0) return fail(SPH_ERR_ARG, "features_step: bad arguments");
  s->lr_refs = 0;  // the learned step's density history no longer applies
  if (s->coarse_sub != substeps) SPH_TRY(ensure_coarse(s, substeps));
  StepOpts o;
  o.scenes = s->d_coarse;
  o.feat = true;
  o.fo = {feat_raw, nullptr, nullptr};
  SPH_TRY(enqueue_step(s, s->stream, nullptr, &o));
  if (ids)
    SPH_CUDA(cudaMemcpyAsync(ids, s->id[s->cp], sizeof(uint32_t) * s->N, cudaMemcpyDeviceToDevice,
                             s->stream), "features_step ids");
  return SPH_OK;
}

int sph_learned_step(SphSystem* s, uint32_t coarse_steps, uint32_t substeps, float tol,
                     uint32_t* fallbacks) {
  if (!s || substeps == 0) return fail(SPH_ERR_ARG, "learned_step: bad arguments");
  if (!s->model_set) return fail(SPH_ERR_STATE, "learned_step: no model (sph_learned_set_model)");
  if (s->coarse_sub != substeps) SPH_TRY(ensure_coarse(s, substeps));
  if (!s->feat) SPH_TRY(dalloc(&s->feat, (size_t)16 * s->N, "features"));
  if (!s->mlp_y) SPH_TRY(dalloc(&s->mlp_y, (size_t)3 * s->N, "corrections"));
  if (!s->bk_vel) SPH_TRY(dalloc(&s->bk_vel, s->N, "checkpoint"));
  if (!s->vstart) SPH_TRY(dalloc(&s->vstart, s->N, "coarse start velocity"));
  if (!s->hist) SPH_TRY(dalloc(&s->hist, s->N, "coarse increments"));
  if (s->lr_refs == 0) s->hist_valid = false;
  std::vector<double> st;
  if (s->lr_refs == 0 && s->stepped) {
    SPH_TRY(scene_stats(s, s->lr_ref[0]));
    s->lr_refs = 1;
  }
  uint32_t fb = 0;
  const float auto_f = (float)(substeps - 1) / (2.f * (float)substeps);
  const float drift = s->drift < 0.f ? auto_f : s->drift;
  const float jerk = s->jerk < 0.f ? auto_f : s->jerk;
  StepOpts o;
  o.scenes = s->d_coarse;
  o.vel_start = s->vstart;
  o.feat = true;
  o.fo = {nullptr, s->feat, s->mlp_aux};
  if (!s->stats_host)
    SPH_CUDA(cudaMallocHost((void**)&s->stats_host, sizeof(double) * 4 * s->S), "stats host buffer");
  // One coarse step on `st`: checkpoint, featured step, MLP, correction, and
  // the per-scene stats copied to the pinned host buffer.  Advances s->cp.
  auto enqueue_coarse = [&](cudaStream_t st) -> int {
    // A step reads pos[cp] and id[cp] and writes the other pair, so only
    // the velocity (overwritten by the force pass) needs a checkpoint.
    SPH_CUDA(cudaMemcpyAsync(s->bk_vel, s->vel[s->cv], sizeof(float4) * s->N, cudaMemcpyDeviceToDevice, st), "checkpoint");
    SPH_TRY(enqueue_step(s, st, nullptr, &o));
    SPH_TRY(sph_mlp_forward_tc(s->mlp_img, s->feat, s->N, s->mlp_y, st));
    k_apply_correction<<<grid_for(s->N, kBlock), kBlock, 0, st>>>(
        s->d_coarse, s->d_poff, s->S, s->N, s->mlp_y, s->mlp_aux + 32, drift, jerk, s->vstart,
        s->vel[1 - s->cv], s->id[s->cp], s->hist, s->hist_valid, s->pos[s->cp], s->vel[s->cv]);
    SPH_CUDA(cudaGetLastError(), "apply correction");
    SPH_CUDA(cudaMemsetAsync(s->stats, 0, sizeof(double) * 4 * s->S, st), "stats clear");
    SPH_TRY(launch_stats(s, st));
    SPH_CUDA(cudaMemcpyAsync(s->stats_host, s->stats, sizeof(double) * 4 * s->S, cudaMemcpyDeviceToHost, st),
             "stats copy");
    return SPH_OK;
  };
  // Without the jerk term (whose history flag changes from step to step)
  // the coarse step is replayed as a CUDA graph, one per buffer parity.
  const bool use_graph = jerk == 0.f;
  const uint64_t key = ((uint64_t)substeps << 32) | (uint64_t)float_bits(drift);
  if (use_graph && s->lgraph_key != key) {
    for (auto& g : s->lgraph)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    s->lgraph_key = key;
  }
  for (uint32_t k = 0; k < coarse_steps; ++k) {
    const int cp0 = s->cp, cv0 = s->cv;
    if (use_graph) {
      if (!s->lgraph[cp0]) {
        if (!s->cap_stream)
          SPH_CUDA(cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking), "capture stream");
        SPH_CUDA(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        const int rc = enqueue_coarse(s->cap_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(s->cap_stream, &g);
        s->cp = cp0;
        if (rc != SPH_OK) {
          if (g) cudaGraphDestroy(g);
          return rc;
        }
        SPH_CUDA(e, "end capture");
        const cudaError_t ie = cudaGraphInstantiate(&s->lgraph[cp0], g, 0);
        cudaGraphDestroy(g);
        SPH_CUDA(ie, "instantiate learned step graph");
      }
      SPH_CUDA(cudaGraphLaunch(s->lgraph[cp0], s->stream), "learned step graph launch");
      s->cp = 1 - cp0;
      s->stepped = true;
      s->inv_ok = false;
    } else {
      SPH_TRY(enqueue_coarse(s->stream));
    }
    s->hist_valid = jerk != 0.f;
    SPH_CUDA(cudaStreamSynchronize(s->stream), "learned step sync");
    st.assign(s->stats_host, s->stats_host + 4 * s->S);
    for (int i = 0; i < s->S; ++i) {
      const double n = s->poff[i + 1] - s->poff[i];
      st[4 * i + 1] = n ? st[4 * i + 1] / n : 0.0;
    }
    // density-deviation check, per scene: the mean density of the step may
    // depart from the linear extrapolation of the last two accepted steps
    // by at most tol (relative), and nothing may be NaN/Inf
    bool ok = true;
    for (int i = 0; i < s->S && ok; ++i) {
      if (st[4 * i + 3] != 0.0 || !(st[4 * i + 1] == st[4 * i + 1])) ok = false;
      if (s->lr_refs > 0 && ok) {
        const double r1 = s->lr_ref[0][4 * i + 1];
        const double pred = s->lr_refs > 1 ? 2.0 * r1 - s->lr_ref[1][4 * i + 1] : r1;
        if (!(fabs(st[4 * i + 1] - pred) <= tol * r1)) ok = false;
      }
    }
    if (!ok) {  // fall back: restore and take `substeps` fine steps
      ++fb;
      s->cp = cp0;
      s->cv = cv0;
      s->hist_valid = false;
      SPH_CUDA(cudaMemcpyAsync(s->vel[cv0], s->bk_vel, sizeof(float4) * s->N, cudaMemcpyDeviceToDevice, s->stream), "restore");
      for (uint32_t q = 0; q < substeps; ++q) SPH_TRY(enqueue_step(s, s->stream));
      SPH_TRY(scene_stats(s, st));
    }
    s->lr_ref[1].swap(s->lr_ref[0]);
    s->lr_ref[0] = st;
    s->lr_refs = s->lr_refs < 2 ? s->lr_refs + 1 : 2;
  }
  if (fallbacks) *fallbacks = fb;
  return SPH_OK;
}

int sph_step_timed(SphSystem* s, float* stage_ms, uint32_t nstages) {
  if (!s || !stage_ms || nstages < (uint32_t)kStepStages)
    return fail(SPH_ERR_ARG, "step_timed: needs room for %d stage times", kStepStages);
  cudaEvent_t ev[kStepStages + 1] = {};
  int rc = SPH_OK;
  for (int k = 0; k <= kStepStages && rc == SPH_OK; ++k)
    rc = cuda_check(cudaEventCreate(&ev[k]), "step_timed: events");
  if (rc == SPH_OK) rc = enqueue_step(s, s->stream, ev);
  if (rc == SPH_OK) rc = cuda_check(cudaEventSynchronize(ev[kStepStages]), "step_timed: sync");
  for (int k = 0; k < kStepStages && rc == SPH_OK; ++k)
    rc = cuda_check(cudaEventElapsedTime(stage_ms + k, ev[k], ev[k + 1]), "step_timed: elapsed");
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  return rc;
}

int sph_get_cells(SphSystem* s, sph_uint2* sortedHash, uint32_t* cellStart, uint32_t* cellEnd,
                  int dst_on_device) {
  if (!s) return fail(SPH_ERR_ARG, "null handle");
  if (!s->stepped) return fail(SPH_ERR_STATE, "get_cells: no step has run");
  uint2* hsh = (uint2*)sortedHash;
  uint32_t *cs = cellStart, *ce = cellEnd;
  uint2* tmp_h = nullptr;
  uint32_t *tmp_s = nullptr, *tmp_e = nullptr;
  if (!dst_on_device) {
    if (sortedHash) SPH_TRY(dalloc(&tmp_h, s->N, "get_cells temp"));
    if (cellStart) SPH_TRY(dalloc(&tmp_s, s->C, "get_cells temp"));
    if (cellEnd) SPH_TRY(dalloc(&tmp_e, s->C, "get_cells temp"));
    hsh = tmp_h;
    cs = tmp_s;
    ce = tmp_e;
  }
  if (hsh)
    k_sorted_hash<<<grid_for(s->N, kBlock), kBlock, 0, s->stream>>>(s->d_scenes, s->d_poff, s->S,
                                                                    s->N, s->pos[s->cp],
                                                                    s->id[s->cp], hsh);
  if (cs || ce)
    k_cell_ranges<<<grid_for(s->C, kBlock), kBlock, 0, s->stream>>>(s->d_scenes, s->d_coff, s->S,
                                                                    s->C, s->start, s->count, cs, ce);
  int rc = cuda_check(cudaGetLastError(), "get_cells kernels");
  if (!dst_on_device && rc == SPH_OK) {
    if (tmp_h) rc = cuda_check(cudaMemcpyAsync(sortedHash, tmp_h, sizeof(uint2) * s->N,
                                               cudaMemcpyDeviceToHost, s->stream), "get_cells copy");
    if (tmp_s && rc == SPH_OK)
      rc = cuda_check(cudaMemcpyAsync(cellStart, tmp_s, sizeof(uint32_t) * s->C,
                                      cudaMemcpyDeviceToHost, s->stream), "get_cells copy");
    if (tmp_e && rc == SPH_OK)
      rc = cuda_check(cudaMemcpyAsync(cellEnd, tmp_e, sizeof(uint32_t) * s->C,
                                      cudaMemcpyDeviceToHost, s->stream), "get_cells copy");
    if (rc == SPH_OK) rc = cuda_check(cudaStreamSynchronize(s->stream), "get_cells sync");
  }
  if (tmp_h) cudaFree(tmp_h);
  if (tmp_s) cudaFree(tmp_s);
  if (tmp_e) cudaFree(tmp_e);
  return rc;
}

int sph_get_fields(SphSystem* s, float* density, float* pressure, int dst_on_device) {
  if (!s) return fail(SPH_ERR_ARG, "null handle");
  const cudaMemcpyKind k = dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (density)
    SPH_CUDA(cudaMemcpyAsync(density, s->dens, sizeof(float) * s->N, k, s->stream), "get_fields");
  if (pressure)
    SPH_CUDA(cudaMemcpyAsync(pressure, s->pres, sizeof(float) * s->N, k, s->stream), "get_fields");
  if (!dst_on_device) SPH_CUDA(cudaStreamSynchronize(s->stream), "get_fields sync");
  return SPH_OK;
}

int sph_stats(SphSystem* s, double* out) {
  if (!s || !out) return fail(SPH_ERR_ARG, "stats: bad arguments");
  SPH_CUDA(cudaMemsetAsync(s->stats, 0, sizeof(double) * 4 * s->S, s->stream), "stats clear");
  SPH_TRY(launch_stats(s, s->stream));
  if (!s->stats_host)
    SPH_CUDA(cudaMallocHost((void**)&s->stats_host, sizeof(double) * 4 * s->S), "stats host buffer");
  SPH_CUDA(cudaMemcpyAsync(s->stats_host, s->stats, sizeof(double) * 4 * s->S,
                           cudaMemcpyDeviceToHost, s->stream), "stats copy");
  SPH_CUDA(cudaStreamSynchronize(s->stream), "stats sync");
  memcpy(out, s->stats_host, sizeof(double) * 4 * s->S);
  for (int i = 0; i < s->S; ++i) {
    const double n = s->poff[i + 1] - s->poff[i];
    out[4 * i + 1] = n ? out[4 * i + 1] / n : 0.0;
  }
  return SPH_OK;
}

int sph_flags(SphSystem* s, uint32_t* flags) {
  if (!s || !flags) return fail(SPH_ERR_ARG, "flags: bad arguments");
  SPH_CUDA(cudaMemcpyAsync(flags, s->flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream),
           "flags copy");
  SPH_CUDA(cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), s->stream), "flags clear");
  return cuda_check(cudaStreamSynchronize(s->stream), "flags sync");
}

}  // extern "C"
