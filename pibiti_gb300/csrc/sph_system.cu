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
//   exclusive scan     count -> start
//   k_scatter_ids      slot[start + rank] = original index
//   k_place            stable position inside the cell = number of smaller
//                      original indices there (the reference's sort is
//                      stable on original order); integrate again and write
//                      the particle there
//   k_density          27-cell poly6 sum (Kernel_Cell.cui:142-199)
//   k_force            27-cell spiky + viscosity, collider, accelerators;
//                      the new velocity is written in sorted order
// so the sorted order (hash, original index) equals the reference's.
#include <cstdio>
#include <cstring>
#include <vector>

#include "sph_device.cuh"
#include "sph_internal.h"

namespace sph {
namespace {

struct __align__(16) SceneDesc {
  SimParams p;
  uint32_t p_off, p_cnt, c_off, c_cnt;
};

constexpr int kBlock = 256;
inline unsigned grid_for(size_t n, int block) { return (unsigned)((n + block - 1) / block); }

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
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

__global__ void __launch_bounds__(kBlock)
k_integrate_count(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S,
                  uint32_t N, const float4* __restrict__ pos, const float4* __restrict__ vel,
                  uint32_t* __restrict__ key, uint32_t* __restrict__ rank,
                  uint32_t* __restrict__ count, uint32_t* __restrict__ flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
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
k_scatter_ids(uint32_t N, const uint32_t* __restrict__ key, const uint32_t* __restrict__ rank,
              const uint32_t* __restrict__ id, const uint32_t* __restrict__ start,
              uint32_t* __restrict__ slot) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  slot[start[key[i]] + rank[i]] = id[i];
}

__global__ void __launch_bounds__(kBlock)
k_place(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
        const float4* __restrict__ pos, const float4* __restrict__ vel,
        const uint32_t* __restrict__ id, const uint32_t* __restrict__ key,
        const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
        const uint32_t* __restrict__ slot, float4* __restrict__ pos_out,
        float4* __restrict__ vel_out, uint32_t* __restrict__ id_out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const uint32_t c = key[i], s0 = start[c], n = count[c], me = id[i];
  uint32_t r = 0;
  for (uint32_t j = s0; j < s0 + n; ++j) r += slot[j] < me;
  const uint32_t dest = s0 + r;
  const SceneDesc& d = sc[S == 1 ? 0 : scene_of(poff, S, i)];
  const float4 x4 = pos[i], v4 = vel[i];
  float3 x = make_float3(x4.x, x4.y, x4.z), v = make_float3(v4.x, v4.y, v4.z);
  integrate(d.p, x, v);
  pos_out[dest] = make_float4(x.x, x.y, x.z, x4.w);
  vel_out[dest] = make_float4(v.x, v.y, v.z, v4.w);
  id_out[dest] = me;
}

// Launch shapes of the two walks: (threads per block, minimum resident
// blocks per SM) pairs; sph_autotune picks one per handle by timing them on
// the handle's own scenes.  Shape 1 (128, 4) is the default, the fastest on
// GB300 for the 1M-particle dam break.
constexpr int kWalkShapes = 3;
constexpr int kWalkBlocks[kWalkShapes] = {64, 128, 256};
constexpr int kDefaultShape = 1;

// Neighbour masks: with 3 * maxParInCell <= 64, the density pass records for
// each particle and each of the 9 neighbour rows (dz, dy) one 64-bit mask
// over the row's candidates (the row's up to 3 cells, each truncated at
// maxParInCell, concatenated in walk order): bit set = squared distance below
// ForceConsts::h2_out (or NaN).  The force pass visits exactly those
// candidates, in the same order, so its sums are unchanged, and skips the
// rest, which the density pass has shown contribute nothing.
constexpr int kRows = 9;
constexpr uint32_t kMaskMaxPerCell = 21;
#ifndef SPH_WALK_MASKS
#define SPH_WALK_MASKS 1  // 0: no mask buffer (saves 72 B per particle)
#endif

__device__ __forceinline__ float h2_out_of(const SimParams& p) {
  return __int_as_float(__float_as_int(__fmul_rn(p.h, p.h)) + 2);
}

template <bool kMask, int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
k_density(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
          const float4* __restrict__ pos, const uint32_t* __restrict__ start,
          const uint32_t* __restrict__ count, float* __restrict__ dens_out,
          float* __restrict__ pres_out, unsigned long long* __restrict__ masks,
          uint32_t* __restrict__ flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
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
      uint32_t bit = 0;
#pragma unroll 1
      for (int x = x0; x <= x1; ++x) {
        const uint32_t c = row + (uint32_t)x;
        uint32_t n = __ldg(count + c);
        if (n > maxpc) {
          trunc = true;
          n = maxpc;
        }
        const uint32_t s0 = __ldg(start + c);
        float cell = 0.f;
        uint32_t m = 0;
        auto cand = [&](uint32_t k) {
          const float4 xj = __ldg(pos + s0 + k);
          const float dx = __fsub_rn(xi.x, xj.x), dy = __fsub_rn(xi.y, xj.y), dz = __fsub_rn(xi.z, xj.z);
          const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
          if (r2 < h2) {
            const float cc = __fsub_rn(h2, r2);
            cell = __fmaf_rn(__fmul_rn(cc, cc), cc, cell);
          }
          if (kMask && !(r2 >= h2_out)) m |= 1u << k;
        };
        // only the particle's own cell holds i
        const uint32_t self = (r == 4 && x == cx) ? i - s0 : 0xffffffffu;
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
        if (kMask) rowmask |= (unsigned long long)m << bit;
        bit += n;
      }
    }
    if (kMask) masks[(size_t)r * N + i] = rowmask;
  }
  if (trunc) atomicOr(flags, 1u);
  const float dens = __fmul_rn(__fmul_rn(sum, p.Poly6Kern), p.particleMass);
  dens_out[i] = dens;
  pres_out[i] = __fmul_rn(__fsub_rn(dens, p.restDensity), p.stiffness);
}

template <bool kMask, int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
k_force(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
        const float4* __restrict__ pos, const float4* __restrict__ vel,
        const float* __restrict__ dens, const float* __restrict__ pres,
        const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
        const unsigned long long* __restrict__ masks, float4* __restrict__ vel_out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const SceneDesc& d = sc[S == 1 ? 0 : scene_of(poff, S, i)];
  const SimParams& p = d.p;
  const float4 xi = pos[i], vi = vel[i];
  const float di = dens[i], pi = pres[i];
  const ForceConsts k = force_consts(p);
  const int3 g = grid_pos(p, xi);
  const int gx = (int)p.gridSize.x, gy = (int)p.gridSize.y, gz = (int)p.gridSize.z;
  const int cx = min(max(g.x, 0), gx - 1), cy = min(max(g.y, 0), gy - 1), cz = min(max(g.z, 0), gz - 1);
  const uint32_t maxpc = p.maxParInCell;
  const int x0 = max(cx - 1, 0), x1 = min(cx + 1, gx - 1);
  float3 F = make_float3(0.f, 0.f, 0.f);
  auto pair = [&](uint32_t j, float3& cell) {
    const float4 xj = __ldg(pos + j);
    const float rx = __fsub_rn(xi.x, xj.x), ry = __fsub_rn(xi.y, xj.y), rz = __fsub_rn(xi.z, xj.z);
    const float dist2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmul_rn(rx, rx)));
    if (!(dist2 >= k.h2_out))
      force_pair_near(k, vi, di, pi, __ldg(vel + j), __ldg(dens + j), __ldg(pres + j), rx, ry, rz,
                      dist2, cell);
  };
  float3 cell = make_float3(0.f, 0.f, 0.f);
  auto flush = [&]() {
    F.x = __fadd_rn(F.x, cell.x);
    F.y = __fadd_rn(F.y, cell.y);
    F.z = __fadd_rn(F.z, cell.z);
    cell = make_float3(0.f, 0.f, 0.f);
  };
  if (kMask) {
    // One loop over every set bit of all 9 row masks, in walk order, so a
    // warp runs max(per-thread neighbour count) iterations rather than the
    // sum over cells of per-cell maxima.  Cell partial sums are flushed
    // into F when the cell changes; skipped (zero) partials leave F as is.
    int r = -1, cur = -1;
    unsigned long long m = 0;
    uint32_t s0 = 0, s1 = 0, s2 = 0, b1 = 0, b2 = 0;
    for (;;) {
      if (m == 0) {
        flush();
        cur = -1;
        for (++r; r < kRows; ++r) {
          const int z = cz + r / 3 - 1, y = cy + r % 3 - 1;
          if (z < 0 || z >= gz || y < 0 || y >= gy) continue;
          m = masks[(size_t)r * N + i];
          if (m) break;
        }
        if (r >= kRows) break;
        const int z = cz + r / 3 - 1, y = cy + r % 3 - 1;
        const uint32_t row = d.c_off + (uint32_t)(z * (int)p.gridSize_yx + y * gx) + (uint32_t)x0;
        const int nc = x1 - x0 + 1;
        const uint32_t n0 = min(__ldg(count + row), maxpc);
        const uint32_t n1 = nc > 1 ? min(__ldg(count + row + 1), maxpc) : 0u;
        s0 = __ldg(start + row);
        s1 = nc > 1 ? __ldg(start + row + 1) : 0u;
        s2 = nc > 2 ? __ldg(start + row + 2) : 0u;
        b1 = n0;
        b2 = n0 + n1;
      }
      const uint32_t b = (uint32_t)(__ffsll((long long)m) - 1);
      m &= m - 1;
      const int c = b >= b2 ? 2 : (b >= b1 ? 1 : 0);
      if (c != cur) {
        flush();
        cur = c;
      }
      const uint32_t j = c == 0 ? s0 + b : (c == 1 ? s1 + (b - b1) : s2 + (b - b2));
      pair(j, cell);
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
        const uint32_t n = min(__ldg(count + c), maxpc);
        const uint32_t s0 = __ldg(start + c);
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

// Per scene, in double: kinetic energy, sum of density, max |rho/rho0-1|,
// non-finite components.  Warps whose lanes share a scene reduce first.
__global__ void k_stats(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S,
                        uint32_t N, const float4* __restrict__ pos, const float4* __restrict__ vel,
                        const float* __restrict__ dens, double* __restrict__ acc) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  int s = -1;
  double ke = 0, rho = 0, dev = 0, bad = 0;
  if (i < N) {
    s = S == 1 ? 0 : scene_of(poff, S, i);
    const SimParams& p = sc[s].p;
    const float4 x = pos[i], v = vel[i];
    const double vx = v.x, vy = v.y, vz = v.z;
    ke = 0.5 * (double)p.particleMass * (vx * vx + vy * vy + vz * vz);
    rho = dens ? (double)dens[i] : 0.0;
    dev = dens ? fabs(rho / (double)p.restDensity - 1.0) : 0.0;
    bad = (double)(!isfinite(x.x) + !isfinite(x.y) + !isfinite(x.z) + !isfinite(v.x) +
                   !isfinite(v.y) + !isfinite(v.z));
    if (!(ke == ke)) ke = 0;
    if (!(dev == dev)) dev = 0;
  }
  const uint32_t peers = __match_any_sync(0xffffffffu, (uint32_t)s);
  if (peers == 0xffffffffu) {
    for (int o = 16; o > 0; o >>= 1) {
      ke += __shfl_xor_sync(0xffffffffu, ke, o);
      rho += __shfl_xor_sync(0xffffffffu, rho, o);
      dev = fmax(dev, __shfl_xor_sync(0xffffffffu, dev, o));
      bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) != 0) return;
  }
  if (s < 0) return;
  atomicAdd(acc + 4 * s + 0, ke);
  atomicAdd(acc + 4 * s + 1, rho);
  atomicMax((unsigned long long*)(acc + 4 * s + 2), (unsigned long long)__double_as_longlong(dev));
  atomicAdd(acc + 4 * s + 3, bad);
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
  uint32_t *count = nullptr, *start = nullptr, *scan_tmp = nullptr;
  float *dens = nullptr, *pres = nullptr;
  unsigned long long* masks = nullptr;  // kRows x N neighbour masks (null: walks without)
  uint32_t* flags = nullptr;
  double* stats = nullptr;
  float4* staging = nullptr;
  int cp = 0;  // pos/id buffer holding the state
  int cv = 0;  // vel buffer holding the state
  bool stepped = false;
  cudaStream_t stream = nullptr;
  bool own_stream = false;  // created here (destroyed here) or borrowed
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // graph_steps steps, keyed by cp at launch
  uint32_t graph_steps = 2;                         // steps per captured graph (even)
  int walk_shape = kDefaultShape;                   // index into kWalkBlocks
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
}

template <bool kMask, int kThreads, int kMinBlocks, class Mark>
void launch_walks_shape(SphSystem* s, cudaStream_t st, int b, int v, Mark& mark) {
  const unsigned g = grid_for(s->N, kThreads);
  k_density<kMask, kThreads, kMinBlocks><<<g, kThreads, 0, st>>>(
      s->d_scenes, s->d_poff, s->S, s->N, s->pos[b], s->start, s->count, s->dens, s->pres,
      s->masks, s->flags);
  mark();
  k_force<kMask, kThreads, kMinBlocks><<<g, kThreads, 0, st>>>(
      s->d_scenes, s->d_poff, s->S, s->N, s->pos[b], s->vel[1 - v], s->dens, s->pres, s->start,
      s->count, s->masks, s->vel[v]);
}

template <bool kMask, class Mark>
void launch_walks(SphSystem* s, cudaStream_t st, int b, int v, Mark& mark) {
  switch (s->walk_shape) {
    case 0: launch_walks_shape<kMask, 64, 8>(s, st, b, v, mark); break;
    case 2: launch_walks_shape<kMask, 256, 2>(s, st, b, v, mark); break;
    default: launch_walks_shape<kMask, 128, 4>(s, st, b, v, mark); break;
  }
}

// Enqueues one step on `st`, advancing s->cp.  With `ev` (kStepStages + 1
// events) an event is recorded before the first stage and after each one.
constexpr int kStepStages = 6;
int enqueue_step(SphSystem* s, cudaStream_t st, cudaEvent_t* ev = nullptr) {
  const unsigned gN = grid_for(s->N, kBlock);
  const int a = s->cp, b = 1 - s->cp, v = s->cv;
  int e = 0;
  auto mark = [&]() {
    if (ev) cudaEventRecord(ev[e++], st);
  };
  mark();
  SPH_CUDA(cudaMemsetAsync(s->count, 0, sizeof(uint32_t) * s->C, st), "step: clear counts");
  k_integrate_count<<<gN, kBlock, 0, st>>>(s->d_scenes, s->d_poff, s->S, s->N, s->pos[a], s->vel[v],
                                           s->key, s->rank, s->count, s->flags);
  mark();
  SPH_TRY(exclusive_scan(s->count, s->start, s->C, s->scan_tmp, st));
  mark();
  k_scatter_ids<<<gN, kBlock, 0, st>>>(s->N, s->key, s->rank, s->id[a], s->start, s->slot);
  mark();
  k_place<<<gN, kBlock, 0, st>>>(s->d_scenes, s->d_poff, s->S, s->N, s->pos[a], s->vel[v], s->id[a],
                                 s->key, s->start, s->count, s->slot, s->pos[b], s->vel[1 - v],
                                 s->id[b]);
  mark();
  if (s->masks)
    launch_walks<true>(s, st, b, v, mark);
  else
    launch_walks<false>(s, st, b, v, mark);
  mark();
  SPH_CUDA(cudaGetLastError(), "step kernels");
  s->cp = b;
  s->stepped = true;
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
                  s->id[0], s->id[1], s->key, s->rank, s->slot, s->count, s->start, s->scan_tmp,
                  s->dens, s->pres, s->masks, s->flags, s->stats, s->staging};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
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
  ALLOC(s->count, c, "cell counts");
  ALLOC(s->start, c, "cell starts");
  ALLOC(s->scan_tmp, scan_scratch_words(c), "scan scratch");
  ALLOC(s->dens, n, "density");
  ALLOC(s->pres, n, "pressure");
  ALLOC(s->flags, 1, "flags");
  bool use_masks = SPH_WALK_MASKS != 0;
  for (uint32_t i = 0; i < count; ++i) use_masks &= scenes[i].maxParInCell <= kMaskMaxPerCell;
  if (use_masks) ALLOC(s->masks, (size_t)kRows * n, "neighbour masks");
  ALLOC(s->stats, 4 * (size_t)count, "stats");
#undef ALLOC
  if (rc == SPH_OK) rc = cuda_check(cudaStreamCreate(&s->stream), "stream");
  s->own_stream = rc == SPH_OK;
  if (rc == SPH_OK) {
    for (int k = 0; k < 2; ++k) {
      cudaMemsetAsync(s->pos[k], 0, sizeof(float4) * n, s->stream);
      cudaMemsetAsync(s->vel[k], 0, sizeof(float4) * n, s->stream);
    }
    cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), s->stream);
    cudaMemsetAsync(s->dens, 0, sizeof(float) * n, s->stream);
    cudaMemsetAsync(s->pres, 0, sizeof(float) * n, s->stream);
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
  const SimParams& o = s->params[scene];
  if (p->numParticles != o.numParticles || p->numCells != o.numCells ||
      p->gridSize.x != o.gridSize.x || p->gridSize.y != o.gridSize.y || p->gridSize.z != o.gridSize.z)
    return fail(SPH_ERR_PARAMS, "set_params: particle count and grid cannot change");
  SPH_TRY(validate_params(*p, true));
  s->params[scene] = *p;
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
  if ((uint64_t)start + count > s->N) return fail(SPH_ERR_ARG, "set_array: range beyond %u particles", s->N);
  if (count == 0) return SPH_OK;
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

int sph_step(SphSystem* s, uint32_t steps) {
  if (!s) return fail(SPH_ERR_ARG, "null handle");
  uint32_t done = 0;
  const uint32_t gs = s->graph_steps;
  if (steps >= gs) {
    if (!s->graph[s->cp]) SPH_TRY(build_graph(s));
    for (; done + gs <= steps; done += gs)
      SPH_CUDA(cudaGraphLaunch(s->graph[s->cp], s->stream), "step graph launch");
  }
  for (; done < steps; ++done) SPH_TRY(enqueue_step(s, s->stream));
  if (steps) s->stepped = true;
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
  if (threads) *threads = (uint32_t)kWalkBlocks[s->walk_shape];
  return SPH_OK;
}

int sph_autotune(SphSystem* s, uint32_t trial_steps, float* ms_per_step, uint32_t* chosen) {
  if (!s || trial_steps == 0) return fail(SPH_ERR_ARG, "autotune: bad arguments");
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
  drop_graphs(s);
  if (chosen) *chosen = (uint32_t)s->walk_shape;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (sp) cudaFree(sp);
  if (sv) cudaFree(sv);
  if (si) cudaFree(si);
  return rc;
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
  k_stats<<<grid_for(s->N, kBlock), kBlock, 0, s->stream>>>(s->d_scenes, s->d_poff, s->S, s->N,
                                                            s->pos[s->cp], s->vel[s->cv],
                                                            s->stepped ? s->dens : nullptr, s->stats);
  SPH_CUDA(cudaGetLastError(), "stats kernel");
  SPH_CUDA(cudaMemcpyAsync(out, s->stats, sizeof(double) * 4 * s->S, cudaMemcpyDeviceToHost, s->stream),
           "stats copy");
  SPH_CUDA(cudaStreamSynchronize(s->stream), "stats sync");
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
