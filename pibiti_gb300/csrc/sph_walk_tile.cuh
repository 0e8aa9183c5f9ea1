// sph_walk_tile.cuh -- the density and force walks with the neighbour
// candidates staged in shared memory.  Included by sph_system.cu inside its
// (anonymous) namespace, after the per-particle walks it falls back to.
//
// A CTA of kThreads threads walks the neighbourhoods of kThreads consecutive
// particles of the sorted order.  Their cells span a small box of the grid
// (one to a few cells when cells are crowded; a run of a cell row when they
// are not); the CTA grows that box by one cell on every side, clipped to the
// grid, and stages the candidates of every cell of it into shared memory:
// the first min(count, maxParInCell) particles of each cell, cell after cell
// in grid order, so each cell's candidates are one contiguous run of slots.
// Every thread then walks its own 27 cells (compDensCell / compForceCell,
// Kernel_Cell.cui:142-261) over those runs instead of over global memory:
// threads whose particles share a cell read the same slots (one broadcast
// shared-memory access per warp), and no per-candidate global address,
// cache tag or L2 round trip remains in the walk.
//
// Density (k_density_tile): the slots hold x, y and z as separate arrays,
// each cell's run padded to an even length with a far-away dummy, so a
// thread evaluates two consecutive candidates with the packed FP32-pair
// instructions of sm_100+ (__fadd2_rn, __fmul2_rn, __ffma2_rn: each half
// rounds exactly as the scalar _rn operation).  The per-cell sum still adds
// the terms one at a time in walk order, so the result is bit-identical to
// the per-particle walk (density_item).
//
// Force (k_force_tile): the slots hold (x, y, z, 1/rho) and (vx, vy, vz, p);
// the thread takes its neighbour-mask bits highest first, as force_item does,
// and finds candidate k of the cell at dx in the slot run of that cell.
//
// A CTA whose box has more than kTileMaxCells cells or whose runs need more
// slots than the launch provides, or (ensembles) whose particles belong to
// two scenes, walks global memory instead (density_item / force_item): the
// results are the same either way.

constexpr int kTileMaxCells = 384;  // box cells a CTA may stage
constexpr float kTileDummy = 3.0e38f;

// Shared-memory state of a staged box.
struct TileHead {
  int x0, y0, z0, bx, by, bz;  // box origin and extent, grid cells
  uint32_t nb;                 // cells in the box
  uint32_t slots;              // staged slots (with padding)
  int scene;                   // the CTA's scene, or -1: walk global memory
  uint32_t trunc;              // a box cell holds more than maxParInCell particles
};

// Head of the CTA's dynamic shared memory; the slot arrays follow it (its
// size is a multiple of 16 bytes, so they start 16-byte aligned).
struct __align__(16) TileTables {
  uint32_t off[kTileMaxCells + 1];  // first slot of each box cell
  uint32_t src[kTileMaxCells];      // first sorted index of each box cell
  uint32_t n[kTileMaxCells];        // candidates of each box cell (count, truncated)
  int red[6 * 32];                  // box reduction, per warp
  uint32_t wsum[32];                // scan, per warp
  TileHead h;
};

// Exclusive scan over the block of one value per thread (kThreads <= 1024).
template <int kThreads>
__device__ __forceinline__ uint32_t tile_block_scan(uint32_t v, uint32_t* wsum, uint32_t* total) {
  constexpr int kWarps = kThreads / 32;
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if ((int)lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < kWarps ? wsum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if ((int)lane >= o) t += y;
    }
    if (lane < kWarps) wsum[lane] = t;
  }
  __syncthreads();
  const uint32_t off = w ? wsum[w - 1] : 0u;
  *total = wsum[kWarps - 1];
  return off + x - v;
}

// The box of the CTA's particles and the slot table of its cells.  `i` is
// the thread's particle (>= N: none), `g` its cell coordinates (clamped into
// the grid).  With kPad, each cell's run is padded to an even length.
// Returns false (uniformly over the block) when the CTA walks global memory.
template <int kThreads, bool kPad>
__device__ bool tile_setup(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S,
                           uint32_t N, uint32_t i0, uint32_t i, int3 g, const uint32_t* __restrict__ start,
                           const uint32_t* __restrict__ count, uint32_t cap, TileTables& t) {
  constexpr int kWarps = kThreads / 32;
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool valid = i < N;
  // box: min and max cell coordinates over the block (warp reductions)
  int v[6] = {valid ? g.x : INT_MAX, valid ? g.y : INT_MAX, valid ? g.z : INT_MAX,
              valid ? -g.x : INT_MAX, valid ? -g.y : INT_MAX, valid ? -g.z : INT_MAX};
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const int m = __reduce_min_sync(0xffffffffu, v[q]);
    if (lane == 0) t.red[6 * w + q] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int m[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) m[q] = t.red[q];
    for (int k = 1; k < kWarps; ++k)
#pragma unroll
      for (int q = 0; q < 6; ++q) m[q] = min(m[q], t.red[6 * k + q]);
    const uint32_t last = min(N - 1, i0 + (uint32_t)kThreads - 1);
    const int s = S == 1 ? 0 : scene_of(poff, S, i0);
    const int s_last = S == 1 ? 0 : scene_of(poff, S, last);
    const SimParams& p = sc[s].p;
    TileHead h;
    h.x0 = max(m[0] - 1, 0);
    h.y0 = max(m[1] - 1, 0);
    h.z0 = max(m[2] - 1, 0);
    h.bx = min(-m[3] + 1, (int)p.gridSize.x - 1) - h.x0 + 1;
    h.by = min(-m[4] + 1, (int)p.gridSize.y - 1) - h.y0 + 1;
    h.bz = min(-m[5] + 1, (int)p.gridSize.z - 1) - h.z0 + 1;
    const long long nb = (long long)h.bx * h.by * h.bz;
    h.nb = (uint32_t)min(nb, (long long)kTileMaxCells + 1);
    h.scene = (s == s_last && nb <= kTileMaxCells) ? s : -1;
    h.slots = 0;
    h.trunc = 0;
    t.h = h;
  }
  __syncthreads();
  const TileHead h = t.h;
  if (h.scene < 0) return false;
  const SceneDesc& d = sc[h.scene];
  const SimParams& p = d.p;
  // per-cell candidate counts, three consecutive box cells per thread at most
  constexpr int kPer = (kTileMaxCells + kThreads - 1) / kThreads;
  const uint32_t c0 = threadIdx.x * kPer;
  uint32_t nloc[kPer], sum = 0;
  bool trunc = false;
  int lx = 0, ly = 0, lz = 0;
  if (c0 < h.nb) {
    lx = (int)(c0 % (uint32_t)h.bx);
    const uint32_t rest = c0 / (uint32_t)h.bx;
    ly = (int)(rest % (uint32_t)h.by);
    lz = (int)(rest / (uint32_t)h.by);
  }
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const uint32_t c = c0 + q;
    nloc[q] = 0;
    if (c < h.nb) {
      const uint32_t gc = d.c_off + (uint32_t)((h.z0 + lz) * (int)p.gridSize_yx +
                                               (h.y0 + ly) * (int)p.gridSize.x + h.x0 + lx);
      const uint32_t n = __ldg(count + gc);
      trunc |= n > p.maxParInCell;
      const uint32_t nt = min(n, p.maxParInCell);
      t.src[c] = __ldg(start + gc);
      t.n[c] = nt;
      nloc[q] = kPad ? (nt + 1u) & ~1u : nt;
      sum += nloc[q];
      if (++lx == h.bx) {
        lx = 0;
        if (++ly == h.by) {
          ly = 0;
          ++lz;
        }
      }
    }
  }
  if (__any_sync(0xffffffffu, trunc) && lane == 0) atomicOr(&t.h.trunc, 1u);
  uint32_t total;
  uint32_t run = tile_block_scan<kThreads>(sum, t.wsum, &total);
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const uint32_t c = c0 + q;
    if (c < h.nb) t.off[c] = run;
    run += nloc[q];
  }
  if (threadIdx.x == 0) {
    t.off[h.nb] = total;
    t.h.slots = total;
  }
  __syncthreads();
  return total <= cap;
}

// ---- density ---------------------------------------------------------------

template <int kThreads>
__global__ void __launch_bounds__(kThreads, 1024 / kThreads)
k_density_tile(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
               const float4* __restrict__ pos, const uint32_t* __restrict__ start,
               const uint32_t* __restrict__ count, float* __restrict__ dens_out,
               float* __restrict__ pres_out, float2* __restrict__ dp_out,
               unsigned long long* __restrict__ masks, uint32_t* __restrict__ flags, uint32_t cap) {
  extern __shared__ __align__(16) unsigned char tile_smem[];
  TileTables& t = *reinterpret_cast<TileTables*>(tile_smem);
  float* sX = reinterpret_cast<float*>(tile_smem + sizeof(TileTables));
  float* sY = sX + cap;
  float* sZ = sY + cap;
  const uint32_t i0 = blockIdx.x * kThreads, i = i0 + threadIdx.x;
  const bool valid = i < N;
  float4 xi = make_float4(0.f, 0.f, 0.f, 0.f);
  int3 g = make_int3(0, 0, 0);
  const SceneDesc& d0 = sc[S == 1 ? 0 : scene_of(poff, S, valid ? i : N - 1)];
  if (valid) {
    xi = __ldg(pos + i);
    const int3 r = grid_pos(d0.p, xi);
    g = make_int3(min(max(r.x, 0), (int)d0.p.gridSize.x - 1), min(max(r.y, 0), (int)d0.p.gridSize.y - 1),
                  min(max(r.z, 0), (int)d0.p.gridSize.z - 1));
  }
  if (!tile_setup<kThreads, true>(sc, poff, S, N, i0, i, g, start, count, cap, t)) {
    if (valid) density_item<true>(sc, poff, S, N, pos, start, count, dens_out, pres_out, dp_out, masks, flags, i);
    return;
  }
  const TileHead h = t.h;
  const SceneDesc& d = sc[h.scene];
  const SimParams& p = d.p;
  // stage: half a warp per cell, one slot per lane (runs are at most 16)
  {
    const uint32_t lane = threadIdx.x & 31, half = lane >> 4, k = lane & 15;
    for (uint32_t c = 2 * (threadIdx.x >> 5) + half; c < h.nb; c += 2 * (kThreads / 32)) {
      const uint32_t o = t.off[c], np = t.off[c + 1] - o;
      if (k < np) {
        float4 x = make_float4(kTileDummy, kTileDummy, kTileDummy, 0.f);
        if (k < t.n[c]) x = __ldg(pos + t.src[c] + k);
        sX[o + k] = x.x;
        sY[o + k] = x.y;
        sZ[o + k] = x.z;
      }
    }
  }
  if (threadIdx.x == 0 && h.trunc) atomicOr(flags, 1u);
  __syncthreads();
  if (!valid) return;
  const int gx = (int)p.gridSize.x, gy = (int)p.gridSize.y, gz = (int)p.gridSize.z;
  const float2 nx = make_float2(-xi.x, -xi.x), ny = make_float2(-xi.y, -xi.y),
               nz = make_float2(-xi.z, -xi.z);
  const float h2 = p.h2, h2o = h2_out_of(p);
  const float2 h2p = make_float2(h2, h2), m1 = make_float2(-1.f, -1.f);
  float sum = 0.f;
  // Two candidates (slots k, k + 1 of one cell's run): r2 and h^2 - r2 as
  // pairs; the cell sum adds the terms in order; mask bits shifted in
  // first-candidate-highest.  kSelf: the run holds slot `ks` of this
  // particle, whose term and bit are dropped.
  auto pairs = [&](auto self_tag, uint32_t k0, uint32_t k1, uint32_t ks, float& cell, uint32_t& m) {
    constexpr bool kSelf = decltype(self_tag)::value;
#pragma unroll 2
    for (uint32_t k = k0; k < k1; k += 2) {
      const float2 X = *reinterpret_cast<const float2*>(sX + k);
      const float2 Y = *reinterpret_cast<const float2*>(sY + k);
      const float2 Z = *reinterpret_cast<const float2*>(sZ + k);
      // x_j - x_i = -(x_i - x_j) exactly, and squares do not see the sign
      const float2 dx = __fadd2_rn(X, nx), dy = __fadd2_rn(Y, ny), dz = __fadd2_rn(Z, nz);
      float2 r2 = __fmul2_rn(dx, dx);
      r2 = __ffma2_rn(dy, dy, r2);
      r2 = __ffma2_rn(dz, dz, r2);
      float2 c = __ffma2_rn(m1, r2, h2p);  // h^2 - r^2, rounded once
      uint32_t b0 = !(r2.x >= h2o), b1 = !(r2.y >= h2o);
      // r^2 >= h^2 (or NaN): no term, as the branch of compDensCell
      c.x = fmaxf(c.x, 0.f);
      c.y = fmaxf(c.y, 0.f);
      if constexpr (kSelf) {
        if (k == ks) {
          c.x = 0.f;
          b0 = 0;
        }
        if (k + 1 == ks) {
          c.y = 0.f;
          b1 = 0;
        }
      }
      const float2 cc = __fmul2_rn(c, c);
      cell = __fmaf_rn(cc.x, c.x, cell);
      cell = __fmaf_rn(cc.y, c.y, cell);
      m = (m << 2) | (b0 << 1) | b1;
    }
  };
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    const int z = g.z + r / 3 - 1, y = g.y + r % 3 - 1;
    unsigned long long rowmask = 0;
    if (z >= 0 && z < gz && y >= 0 && y < gy) {
      const int lrow = ((z - h.z0) * h.by + (y - h.y0)) * h.bx - h.x0;
#pragma unroll 1
      for (int f = 0; f < 3; ++f) {
        const int x = g.x - 1 + f;
        if (x < 0 || x >= gx) continue;
        const uint32_t c = (uint32_t)(lrow + x);
        const uint32_t o0 = t.off[c], o1 = t.off[c + 1], n = t.n[c];
        float cell = 0.f;
        uint32_t m = 0;
        if (r == 4 && f == 1) {
          const uint32_t ks = i - t.src[c];  // this particle's slot, if a candidate
          const uint32_t kss = ks < n ? o0 + ks : 0xffffffffu;
          pairs(std::true_type{}, o0, o1, kss, cell, m);
        } else {
          pairs(std::false_type{}, o0, o1, 0u, cell, m);
        }
        sum = __fadd_rn(sum, cell);
        // m: one bit per slot of the run, slot o0 highest; drop the dummy
        const uint32_t np = o1 - o0;
        uint32_t field = np ? (m << (16 - np)) & 0xFFFFu : 0u;
        field &= (0xFFFFu << (16 - n)) & 0xFFFFu;
        rowmask |= (unsigned long long)field << (16 * (2 - f));
      }
    }
    masks[(size_t)r * N + i] = rowmask;
  }
  const float dens = __fmul_rn(__fmul_rn(sum, p.Poly6Kern), p.particleMass);
  const float pres = __fmul_rn(__fsub_rn(dens, p.restDensity), p.stiffness);
  dens_out[i] = dens;
  pres_out[i] = pres;
  dp_out[i] = make_float2(__frcp_rn(dens), pres);
}

// ---- force -------------------------------------------------------------------

template <int kThreads>
__global__ void __launch_bounds__(kThreads, 512 / kThreads)
k_force_tile(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
             const float4* __restrict__ pos, const float4* __restrict__ vel,
             const float* __restrict__ dens, const float2* __restrict__ dp,
             const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
             const unsigned long long* __restrict__ masks, float4* __restrict__ vel_out, uint32_t cap) {
  extern __shared__ __align__(16) unsigned char tile_smem[];
  TileTables& t = *reinterpret_cast<TileTables*>(tile_smem);
  float4* sP = reinterpret_cast<float4*>(tile_smem + sizeof(TileTables));
  float4* sV = sP + cap;
  const uint32_t i0 = blockIdx.x * kThreads;
  const uint32_t i = regrouped_particle<kThreads>(sc, poff, S, N, pos);
  const bool valid = i < N;
  float4 xi = make_float4(0.f, 0.f, 0.f, 0.f);
  int3 g = make_int3(0, 0, 0);
  const SceneDesc& d0 = sc[S == 1 ? 0 : scene_of(poff, S, valid ? i : N - 1)];
  if (valid) {
    xi = __ldg(pos + i);
    const int3 r = grid_pos(d0.p, xi);
    g = make_int3(min(max(r.x, 0), (int)d0.p.gridSize.x - 1), min(max(r.y, 0), (int)d0.p.gridSize.y - 1),
                  min(max(r.z, 0), (int)d0.p.gridSize.z - 1));
  }
  const FeatOut no_feat = {nullptr, nullptr, nullptr};
  if (!tile_setup<kThreads, false>(sc, poff, S, N, i0, i, g, start, count, cap, t)) {
    if (valid) force_item<true, false>(sc, poff, S, N, pos, vel, dens, dp, start, count, masks, vel_out, no_feat, i);
    return;
  }
  const TileHead h = t.h;
  const SceneDesc& d = sc[h.scene];
  const SimParams& p = d.p;
  // stage: half a warp per cell, one slot per lane
  {
    const uint32_t lane = threadIdx.x & 31, half = lane >> 4, k = lane & 15;
    for (uint32_t c = 2 * (threadIdx.x >> 5) + half; c < h.nb; c += 2 * (kThreads / 32)) {
      const uint32_t o = t.off[c];
      if (k < t.n[c]) {
        const uint32_t j = t.src[c] + k;
        const float4 x = __ldg(pos + j), v = __ldg(vel + j);
        const float2 q = __ldg(dp + j);
        sP[o + k] = make_float4(x.x, x.y, x.z, q.x);
        sV[o + k] = make_float4(v.x, v.y, v.z, q.y);
      }
    }
  }
  __syncthreads();
  if (!valid) return;
  const float4 vi = __ldg(vel + i);
  const float2 dpi = __ldg(dp + i);
  const float inv_di = dpi.x, pi = dpi.y;
  const ForceConsts k = force_consts(p);
  const int gx = (int)p.gridSize.x, gy = (int)p.gridSize.y, gz = (int)p.gridSize.z;
  float3 F = make_float3(0.f, 0.f, 0.f), cell = make_float3(0.f, 0.f, 0.f);
  auto flush = [&]() {
    F.x = __fadd_rn(F.x, cell.x);
    F.y = __fadd_rn(F.y, cell.y);
    F.z = __fadd_rn(F.z, cell.z);
    cell = make_float3(0.f, 0.f, 0.f);
  };
  auto term = [&](uint32_t s, float3& f) -> bool {
    const float4 a = sP[s], b = sV[s];
    const float rx = __fsub_rn(xi.x, a.x), ry = __fsub_rn(xi.y, a.y), rz = __fsub_rn(xi.z, a.z);
    const float dist2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmul_rn(rx, rx)));
    return force_term(k, vi, inv_di, pi, b, a.w, b.w, rx, ry, rz, dist2, f);
  };
  unsigned long long mnext = masks[i];
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    unsigned long long m = mnext;
    if (r + 1 < kRows) mnext = masks[(size_t)(r + 1) * N + i];
    const int z = g.z + r / 3 - 1, y = g.y + r % 3 - 1;
    if (!m || z < 0 || z >= gz || y < 0 || y >= gy) continue;
    const int c1 = ((z - h.z0) * h.by + (y - h.y0)) * h.bx + (g.x - h.x0);
    // first slot of the cell at dx = -1, 0, +1 (a field outside the grid has no bit)
    const uint32_t o0 = g.x > 0 ? t.off[c1 - 1] : 0u;
    const uint32_t o1 = t.off[c1];
    const uint32_t o2 = g.x + 1 < gx ? t.off[c1 + 1] : 0u;
    auto slot_of = [&](int b, int f) { return (f == 0 ? o0 : (f == 1 ? o1 : o2)) + mask_cand(b); };
    int cur = -1;
    while (m) {
      const int ba = 63 - __clzll((long long)m);
      m ^= 1ull << ba;
      const bool two = m != 0;
      const int bb = two ? 63 - __clzll((long long)m) : ba;
      if (two) m ^= 1ull << bb;
      const int fa = mask_field(ba), fb = mask_field(bb);
      float3 ta, tb;
      const bool ina = term(slot_of(ba, fa), ta);
      const bool inb = term(slot_of(bb, fb), tb);
      if (fa != cur) {
        flush();
        cur = fa;
      }
      if (ina) {
        cell.x = __fadd_rn(cell.x, ta.x);
        cell.y = __fadd_rn(cell.y, ta.y);
        cell.z = __fadd_rn(cell.z, ta.z);
      }
      if (two) {
        if (fb != cur) {
          flush();
          cur = fb;
        }
        if (inb) {
          cell.x = __fadd_rn(cell.x, tb.x);
          cell.y = __fadd_rn(cell.y, tb.y);
          cell.z = __fadd_rn(cell.z, tb.z);
        }
      }
    }
    flush();
  }
  const float3 add = velocity_increment(p, F, xi, vi);
  vel_out[i] = make_float4(__fadd_rn(vi.x, add.x), __fadd_rn(vi.y, add.y), __fadd_rn(vi.z, add.z),
                           __fadd_rn(vi.w, 0.f));
}

// ---- density, second form: interleaved candidate pairs ------------------------
// Slots in pairs: pair q holds (x, x', y, y') in one float4 and (z, z') in one
// float2, so a thread loads two candidates with two shared-memory loads.  The
// capacity is a compile-time constant (the z array sits at a fixed offset).
// Per pair of candidates: the squared distances and h^2 - r^2 as FP32 pairs,
// max(h^2 - r^2, 0) by a saturating FMA (exact for h^2 <= 1: a positive
// difference below 1 is unchanged, a negative one or NaN becomes +0), and
// the mask bits from the sign bits of h2_out - r^2 shifted in with funnel
// shifts (sign set = outside; the field keeps the complement, so a NaN
// distance, whose difference has a clear sign bit, stays in the mask as
// !(r2 >= h2_out) keeps it).  A squared distance equal to h2_out also stays
// in: the mask only has to hold every pair the force pass can use, and the
// force term itself rejects r >= h.

__device__ __forceinline__ float fma_sat(float a, float b, float c) {
  float d;
  asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

template <int kThreads, uint32_t kPairs>
__global__ void __launch_bounds__(kThreads, 1024 / kThreads)
k_density_pairs(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
                const float4* __restrict__ pos, const uint32_t* __restrict__ start,
                const uint32_t* __restrict__ count, float* __restrict__ dens_out,
                float* __restrict__ pres_out, float2* __restrict__ dp_out,
                unsigned long long* __restrict__ masks, uint32_t* __restrict__ flags) {
  extern __shared__ __align__(16) unsigned char tile_smem[];
  TileTables& t = *reinterpret_cast<TileTables*>(tile_smem);
  float4* sXY = reinterpret_cast<float4*>(tile_smem + sizeof(TileTables));
  float2* sZ = reinterpret_cast<float2*>(sXY + kPairs);
  const uint32_t i0 = blockIdx.x * kThreads, i = i0 + threadIdx.x;
  const bool valid = i < N;
  float4 xi = make_float4(0.f, 0.f, 0.f, 0.f);
  int3 g = make_int3(0, 0, 0);
  const SceneDesc& d0 = sc[S == 1 ? 0 : scene_of(poff, S, valid ? i : N - 1)];
  if (valid) {
    xi = __ldg(pos + i);
    const int3 r = grid_pos(d0.p, xi);
    g = make_int3(min(max(r.x, 0), (int)d0.p.gridSize.x - 1), min(max(r.y, 0), (int)d0.p.gridSize.y - 1),
                  min(max(r.z, 0), (int)d0.p.gridSize.z - 1));
  }
  // the saturating form needs h^2 <= 1 (uniform: one scene per staged block)
  const bool ok = tile_setup<kThreads, true>(sc, poff, S, N, i0, i, g, start, count, 2 * kPairs, t) &&
                  sc[t.h.scene].p.h2 <= 1.f;
  if (!ok) {
    if (valid) density_item<true>(sc, poff, S, N, pos, start, count, dens_out, pres_out, dp_out, masks, flags, i);
    return;
  }
  const TileHead h = t.h;
  const SimParams& p = sc[h.scene].p;
  {
    float* xy = reinterpret_cast<float*>(sXY);
    float* zz = reinterpret_cast<float*>(sZ);
    const uint32_t lane = threadIdx.x & 31, half = lane >> 4, k = lane & 15;
    for (uint32_t c = 2 * (threadIdx.x >> 5) + half; c < h.nb; c += 2 * (kThreads / 32)) {
      const uint32_t o = t.off[c], np = t.off[c + 1] - o;
      if (k < np) {
        float4 x = make_float4(kTileDummy, kTileDummy, kTileDummy, 0.f);
        if (k < t.n[c]) x = __ldg(pos + t.src[c] + k);
        const uint32_t s = o + k, q = s >> 1, e = s & 1;
        xy[4 * q + e] = x.x;
        xy[4 * q + 2 + e] = x.y;
        zz[2 * q + e] = x.z;
      }
    }
  }
  if (threadIdx.x == 0 && h.trunc) atomicOr(flags, 1u);
  __syncthreads();
  if (!valid) return;
  const int gx = (int)p.gridSize.x, gy = (int)p.gridSize.y, gz = (int)p.gridSize.z;
  const float2 nx = make_float2(-xi.x, -xi.x), ny = make_float2(-xi.y, -xi.y),
               nz = make_float2(-xi.z, -xi.z);
  const float h2 = p.h2, h2o = h2_out_of(p);
  const float2 h2o2 = make_float2(h2o, h2o), m1 = make_float2(-1.f, -1.f);
  float sum = 0.f;
  // pairs q0..q1-1 of one cell's run; `out` collects one bit per slot, the
  // first slot highest, set when the candidate lies beyond h2_out
  auto run = [&](auto self_tag, uint32_t q0, uint32_t q1, uint32_t qs, uint32_t es, float& cell,
                 uint32_t& out) {
    constexpr bool kSelf = decltype(self_tag)::value;
#pragma unroll 2
    for (uint32_t q = q0; q < q1; ++q) {
      const float4 a = sXY[q];
      const float2 zq = sZ[q];
      const float2 dx = __fadd2_rn(make_float2(a.x, a.y), nx);
      const float2 dy = __fadd2_rn(make_float2(a.z, a.w), ny);
      const float2 dz = __fadd2_rn(zq, nz);
      float2 r2 = __fmul2_rn(dx, dx);
      r2 = __ffma2_rn(dy, dy, r2);
      r2 = __ffma2_rn(dz, dz, r2);
      const float2 e = __ffma2_rn(m1, r2, h2o2);
      float c0 = fma_sat(-1.f, r2.x, h2), c1 = fma_sat(-1.f, r2.y, h2);
      uint32_t u0 = __float_as_uint(e.x), u1 = __float_as_uint(e.y);
      if constexpr (kSelf) {
        if (q == qs) {  // this particle: no term, no bit
          if (es == 0) {
            c0 = 0.f;
            u0 = 0x80000000u;
          } else {
            c1 = 0.f;
            u1 = 0x80000000u;
          }
        }
      }
      const float2 cc = __fmul2_rn(make_float2(c0, c1), make_float2(c0, c1));
      cell = __fmaf_rn(cc.x, c0, cell);
      cell = __fmaf_rn(cc.y, c1, cell);
      out = __funnelshift_l(u0, out, 1);
      out = __funnelshift_l(u1, out, 1);
    }
  };
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    const int z = g.z + r / 3 - 1, y = g.y + r % 3 - 1;
    unsigned long long rowmask = 0;
    if (z >= 0 && z < gz && y >= 0 && y < gy) {
      const int lrow = ((z - h.z0) * h.by + (y - h.y0)) * h.bx - h.x0;
#pragma unroll 1
      for (int f = 0; f < 3; ++f) {
        const int x = g.x - 1 + f;
        if (x < 0 || x >= gx) continue;
        const uint32_t c = (uint32_t)(lrow + x);
        const uint32_t o0 = t.off[c], o1 = t.off[c + 1], n = t.n[c];
        float cell = 0.f;
        uint32_t out = 0;
        if (r == 4 && f == 1) {
          const uint32_t ks = i - t.src[c];  // this particle's place in the cell
          const uint32_t s = ks < n ? o0 + ks : 0xffffffffu;
          run(std::true_type{}, o0 >> 1, o1 >> 1, s >> 1, s & 1, cell, out);
        } else {
          run(std::false_type{}, o0 >> 1, o1 >> 1, 0xffffffffu, 0u, cell, out);
        }
        sum = __fadd_rn(sum, cell);
        // in-bits of the run's real candidates, candidate 0 at bit 15
        const uint32_t np = o1 - o0;
        uint32_t field = np ? ((~out << (16 - np)) & (0xFFFFu << (16 - n))) & 0xFFFFu : 0u;
        rowmask |= (unsigned long long)field << (16 * (2 - f));
      }
    }
    masks[(size_t)r * N + i] = rowmask;
  }
  const float dens = __fmul_rn(__fmul_rn(sum, p.Poly6Kern), p.particleMass);
  const float pres = __fmul_rn(__fsub_rn(dens, p.restDensity), p.stiffness);
  dens_out[i] = dens;
  pres_out[i] = pres;
  dp_out[i] = make_float2(__frcp_rn(dens), pres);
}

// ---- force, by cell fields ----------------------------------------------------
// The masked walk of force_item, taken one cell (one 16-bit field of a row
// mask) at a time: the cell's start is loaded once, its set bits are taken
// highest first with 32-bit operations, and its partial sum is added to the
// total when its bits are done (a cell without a set bit would add +0, which
// changes nothing, so it is skipped).
// With kFeat (the learned step's coarse step) it also accumulates the pair
// sums of the 16 features in the same walk order as force_item and writes
// them (feature_out), so the features equal the row walk's.
template <int kThreads, int kMinBlocks, bool kFeat>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
k_force_fields(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
               const float4* __restrict__ pos, const float4* __restrict__ vel,
               const float2* __restrict__ dp, const uint32_t* __restrict__ start,
               const unsigned long long* __restrict__ masks, float4* __restrict__ vel_out,
               const float* __restrict__ dens, FeatOut fo) {
  const uint32_t i = regrouped_particle<kThreads>(sc, poff, S, N, pos);
  if (i >= N) return;
  const SceneDesc& d = sc[S == 1 ? 0 : scene_of(poff, S, i)];
  const SimParams& p = d.p;
  const float4 xi = __ldg(pos + i), vi = __ldg(vel + i);
  const float2 dpi = __ldg(dp + i);
  const float inv_di = dpi.x, pi = dpi.y;
  const ForceConsts k = force_consts(p);
  const int3 g0 = grid_pos(p, xi);
  const int gx = (int)p.gridSize.x, gy = (int)p.gridSize.y, gz = (int)p.gridSize.z;
  const int cx = min(max(g0.x, 0), gx - 1), cy = min(max(g0.y, 0), gy - 1), cz = min(max(g0.z, 0), gz - 1);
  // x and y as FP32 pairs (force_term_xy); xi - xj as fma(xj, -1, xi)
  const float2 xi_xy = make_float2(xi.x, xi.y), vi_xy = make_float2(vi.x, vi.y);
  float2 F_xy = make_float2(0.f, 0.f);
  float F_z = 0.f;
  FeatAcc fa;
  const float inv_h = kFeat ? 1.f / p.h : 0.f;
  unsigned long long mnext = masks[i];
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    const unsigned long long m = mnext;
    if (r + 1 < kRows) mnext = masks[(size_t)(r + 1) * N + i];
    if (!m) continue;
    const int z = cz + r / 3 - 1, y = cy + r % 3 - 1;
    const int row = z * (int)p.gridSize_yx + y * gx + cx;  // the cell at dx = 0
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
      uint32_t bits = (uint32_t)(m >> (16 * (2 - f))) & 0xFFFFu;
      if (!bits) continue;
      // the cell at dx = f - 1 (a field outside the grid holds no bit); its
      // index is formed before the pointer, so the cell at dx = -1 of the
      // grid's first cell never becomes a 2^32-element pointer offset
      const uint32_t c = d.c_off + (uint32_t)(row + f - 1);
      const uint32_t s0 = __ldg(start + c) + 15u;
      float2 cell_xy = make_float2(0.f, 0.f);
      float cell_z = 0.f;
      do {
        const int b = 31 - __clz(bits);
        bits ^= 1u << b;
        const uint32_t j = s0 - (uint32_t)b;  // candidate 15 - b
        const float4 xj = __ldg(pos + j), vj = __ldg(vel + j);
        const float2 dpj = __ldg(dp + j);
        const float2 r_xy = __ffma2_rn(make_float2(xj.x, xj.y), make_float2(-1.f, -1.f), xi_xy);
        const float rz = __fsub_rn(xi.z, xj.z);
        const float dist2 = __fmaf_rn(rz, rz, __fmaf_rn(r_xy.y, r_xy.y, __fmul_rn(r_xy.x, r_xy.x)));
        float2 t_xy;
        float t_z;
        if (force_term_xy(k, vi_xy, vi.z, inv_di, pi, vj, dpj.x, dpj.y, r_xy, rz, dist2, t_xy, t_z)) {
          cell_xy = __fadd2_rn(cell_xy, t_xy);
          cell_z = __fadd_rn(cell_z, t_z);
        }
        if (kFeat) feat_add(fa, k, inv_h, vi, vj, r_xy.x, r_xy.y, rz, dist2);
      } while (bits);
      F_xy = __fadd2_rn(F_xy, cell_xy);
      F_z = __fadd_rn(F_z, cell_z);
    }
  }
  const float3 add = velocity_increment(p, make_float3(F_xy.x, F_xy.y, F_z), xi, vi);
  vel_out[i] = make_float4(__fadd_rn(vi.x, add.x), __fadd_rn(vi.y, add.y), __fadd_rn(vi.z, add.z),
                           __fadd_rn(vi.w, 0.f));
  if (kFeat) feature_out(p, fa, make_float3(F_xy.x, F_xy.y, F_z), xi, vi, pi, dens[i], fo, i);
}

// ---- force, warp-cooperative by rows --------------------------------------------
// The masked walk one neighbour row (dz, dy) at a time, with the pair terms
// of the whole warp evaluated together.  For each row:
//   1. every thread lists its pairs of the row in walk order (candidate
//      index, owning lane, x field) in the warp's part of shared memory, at
//      an offset from a warp prefix sum of the threads' pair counts;
//   2. the warp evaluates the list 32 pairs at a time, each lane taking any
//      thread's pair (the owner's position, velocity, 1/rho and pressure come
//      from the warp's particle table), and writes the term to the list's
//      result slot (zero when r >= h);
//   3. every thread adds its own results in list order, flushing the cell's
//      partial sum into its total where the x field changes.
// Step 2 keeps all lanes busy however unevenly the pairs fall over the
// threads, which is what limits the one-thread-per-particle walk when cells
// hold one or two neighbours each; steps 1 and 3 are a few instructions per
// pair.  The sums are the per-thread walk's, in the same order.  A row whose
// warp total exceeds kCoopCap pairs is walked one thread per particle.
constexpr int kCoopCap = 256;

template <int kThreads>
__global__ void __launch_bounds__(kThreads, 1024 / kThreads)
k_force_coop(const SceneDesc* __restrict__ sc, const uint32_t* __restrict__ poff, int S, uint32_t N,
             const float4* __restrict__ pos, const float4* __restrict__ vel,
             const float2* __restrict__ dp, const uint32_t* __restrict__ start,
             const unsigned long long* __restrict__ masks, float4* __restrict__ vel_out) {
  constexpr int kW = kThreads / 32;
  __shared__ uint2 s_ent[kW][kCoopCap];     // (candidate index, owner lane | field << 8)
  __shared__ float4 s_res[kW][kCoopCap];    // pair term, w unused
  __shared__ float4 s_px[kW][32], s_pv[kW][32];  // (x, y, z, 1/rho), (vx, vy, vz, p) per lane
  const uint32_t i = regrouped_particle<kThreads>(sc, poff, S, N, pos);
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool valid = i < N;
  // a warp whose threads all have no particle leaves together
  if (!__any_sync(0xffffffffu, valid)) return;
  const SceneDesc& d = sc[S == 1 ? 0 : scene_of(poff, S, valid ? i : N - 1)];
  const SimParams& p = d.p;
  float4 xi = make_float4(0.f, 0.f, 0.f, 0.f), vi = xi;
  float2 dpi = make_float2(0.f, 0.f);
  if (valid) {
    xi = __ldg(pos + i);
    vi = __ldg(vel + i);
    dpi = __ldg(dp + i);
  }
  s_px[w][lane] = make_float4(xi.x, xi.y, xi.z, dpi.x);
  s_pv[w][lane] = make_float4(vi.x, vi.y, vi.z, dpi.y);
  const ForceConsts k = force_consts(p);
  const int3 g0 = grid_pos(p, xi);
  const int gx = (int)p.gridSize.x, gy = (int)p.gridSize.y, gz = (int)p.gridSize.z;
  const int cx = min(max(g0.x, 0), gx - 1), cy = min(max(g0.y, 0), gy - 1), cz = min(max(g0.z, 0), gz - 1);
  float3 F = make_float3(0.f, 0.f, 0.f);
  auto add = [](float3& a, float x, float y, float z) {
    a.x = __fadd_rn(a.x, x);
    a.y = __fadd_rn(a.y, y);
    a.z = __fadd_rn(a.z, z);
  };
  unsigned long long mnext = valid ? masks[i] : 0ull;
#pragma unroll 1
  for (int r = 0; r < kRows; ++r) {
    const unsigned long long m = mnext;
    if (r + 1 < kRows) mnext = valid ? masks[(size_t)(r + 1) * N + i] : 0ull;
    // pairs of this row per thread; warp prefix sum and total
    const uint32_t np = (uint32_t)__popcll((long long)m);
    uint32_t incl = np;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31), base = incl - np;
    if (total == 0) continue;
    const int row = (cz + r / 3 - 1) * (int)p.gridSize_yx + (cy + r % 3 - 1) * gx + cx;  // dx = 0
    if (total > (uint32_t)kCoopCap) {
      // a crowded row: one thread per particle, cell field by cell field
#pragma unroll 1
      for (int f = 0; f < 3; ++f) {
        uint32_t bits = (uint32_t)(m >> (16 * (2 - f))) & 0xFFFFu;
        if (!bits) continue;
        const uint32_t s0 = __ldg(start + (d.c_off + (uint32_t)(row + f - 1))) + 15u;
        float3 cell = make_float3(0.f, 0.f, 0.f);
        do {
          const int b = 31 - __clz(bits);
          bits ^= 1u << b;
          const uint32_t j = s0 - (uint32_t)b;
          const float4 xj = __ldg(pos + j), vj = __ldg(vel + j);
          const float2 dpj = __ldg(dp + j);
          const float rx = __fsub_rn(xi.x, xj.x), ry = __fsub_rn(xi.y, xj.y), rz = __fsub_rn(xi.z, xj.z);
          const float dist2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmul_rn(rx, rx)));
          float3 t;
          if (force_term(k, vi, dpi.x, dpi.y, vj, dpj.x, dpj.y, rx, ry, rz, dist2, t)) add(cell, t.x, t.y, t.z);
        } while (bits);
        add(F, cell.x, cell.y, cell.z);
      }
      continue;
    }
    // 1. list this thread's pairs of the row, walk order
    uint32_t q = base;
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
      uint32_t bits = (uint32_t)(m >> (16 * (2 - f))) & 0xFFFFu;
      if (!bits) continue;
      const uint32_t s0 = __ldg(start + (d.c_off + (uint32_t)(row + f - 1))) + 15u;
      do {
        const int b = 31 - __clz(bits);
        bits ^= 1u << b;
        s_ent[w][q++] = make_uint2(s0 - (uint32_t)b, lane | ((uint32_t)f << 8));
      } while (bits);
    }
    __syncwarp();
    // 2. all pair terms of the warp's row
#pragma unroll 1
    for (uint32_t e = lane; e < total; e += 32) {
      const uint2 en = s_ent[w][e];
      const uint32_t j = en.x, own = en.y & 31u;
      const float4 a = s_px[w][own], b = s_pv[w][own];
      const float4 xj = __ldg(pos + j), vj = __ldg(vel + j);
      const float2 dpj = __ldg(dp + j);
      const float rx = __fsub_rn(a.x, xj.x), ry = __fsub_rn(a.y, xj.y), rz = __fsub_rn(a.z, xj.z);
      const float dist2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmul_rn(rx, rx)));
      float3 t;
      const bool in = force_term(k, b, a.w, b.w, vj, dpj.x, dpj.y, rx, ry, rz, dist2, t);
      // r >= h: no term (+0 leaves a partial sum unchanged)
      s_res[w][e] = in ? make_float4(t.x, t.y, t.z, 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncwarp();
    // 3. this thread's terms in order, the cell sum flushed at each field change
    if (np) {
      float3 cell = make_float3(0.f, 0.f, 0.f);
      uint32_t cur = s_ent[w][base].y >> 8;
#pragma unroll 1
      for (uint32_t e = base; e < base + np; ++e) {
        const uint32_t fld = s_ent[w][e].y >> 8;
        if (fld != cur) {
          add(F, cell.x, cell.y, cell.z);
          cell = make_float3(0.f, 0.f, 0.f);
          cur = fld;
        }
        const float4 t = s_res[w][e];
        add(cell, t.x, t.y, t.z);
      }
      add(F, cell.x, cell.y, cell.z);
    }
    __syncwarp();
  }
  if (!valid) return;
  const float3 dv = velocity_increment(p, F, xi, vi);
  vel_out[i] = make_float4(__fadd_rn(vi.x, dv.x), __fadd_rn(vi.y, dv.y), __fadd_rn(vi.z, dv.z),
                           __fadd_rn(vi.w, 0.f));
}
