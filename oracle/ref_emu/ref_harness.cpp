/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY (part of the oracle).
 *
 * Runs the reference's own SPH kernels and radix sort on the host CPU.  The
 * kernels themselves come unmodified from the reference tree (System.cu
 * lines 1-548, radixsort_kernel.cu lines 1-432), compiled by g++ with
 * emu_prelude.h force-included; see build_ref.sh.  This file supplies what
 * nvcc and the GPU would: a block/thread launcher (a fibre per CUDA thread
 * for kernels that use __syncthreads), texture binding, and host-side copies
 * of the reference's `extern "C"` wrappers (System.cu:653-756,
 * radixsort_kernel.cu:445-472) with GL buffer ids replaced by host pointers.
 *
 * It also exposes the reference's scene loader (Scene.cpp, Scene_Load.cpp
 * with TinyXML), so the parameter derivations can be checked byte for byte.
 *
 * Only tests/golden/make_golden.py and the not-gpu tests load the resulting
 * oracle/_ref/libref_emu.so; nothing in the product does.
 */
#include <ucontext.h>
#include <cstdio>
#include <cstring>
#include <functional>
#include <vector>

#include "Params.cuh"
#include "radixsort.cuh"

/* ---- CUDA built-in variables and dynamic shared memory ---------------- */
uint3 threadIdx;
uint3 blockIdx;
dim3 blockDim;
dim3 gridDim;
/* `extern __shared__ uint sRadixSum[]` (radixsort_kernel.cu:55); the largest
   request is PREFIX_GRFSIZE = (16384/16 + 2*192) uints. */
uint sRadixSum[8192];

/* ---- symbols defined by the reference translation units --------------- */
extern SimParams par;
extern texture<float4, 1, cudaReadModeElementType> oldPosTex, oldVelTex;
extern texture<uint2, 1, cudaReadModeElementType> particleHashTex;
extern texture<uint, 1, cudaReadModeElementType> cellStartTex;
extern texture<float, 1, cudaReadModeElementType> pressureTex, densityTex, dyeColorTex;

void integrateD(float4* newPos, float4* newVel, float4* oldPos, float4* oldVel);
void calcHashD(float4* pos, uint2* particleHash);
void reorderD(uint2* particleHash, uint* cellStart, float4* oldPos, float4* oldVel,
              float4* sortedPos, float4* sortedVel);
void computeDensityD(float4* clr, float4* oldPos, float* pressure, float* density,
                     uint2* particleHash, uint* cellStart);
void computeForceD(float4* newPos, float4* newVel, float4* oldPos, float4* oldVel, float4* clr,
                   float* pressure, float* density, float* dyeColor, uint2* particleHash,
                   uint* cellStart);
void RadixSum(KeyValuePair* pData, uint elements, uint elements_rounded_to_3072, uint shift);
void RadixPrefixSum();
void RadixAddOffsetsAndShuffle(KeyValuePair* pSrc, KeyValuePair* pDst, uint elements,
                               uint elements_rounded_to_3072, int shift);

/* ---- launcher ---------------------------------------------------------- */
namespace {

struct Fibre {
  ucontext_t ctx;
  uint3 tid;
  bool done;
};

ucontext_t g_sched;
Fibre* g_cur = nullptr;
const std::function<void()>* g_body = nullptr;
constexpr size_t kStack = 64 * 1024;

void fibre_entry() {
  (*g_body)();
  g_cur->done = true;
}

/* Every thread of a block runs as a fibre; __syncthreads switches back here.
   Each round resumes every live fibre once, so all of them reach the same
   barrier before any passes it. */
void launch_sync(dim3 grid, dim3 block, const std::function<void()>& body) {
  const unsigned nt = block.x * block.y * block.z;
  std::vector<Fibre> f(nt);
  std::vector<char> stacks((size_t)nt * kStack);
  gridDim = grid;
  blockDim = block;
  g_body = &body;
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        blockIdx = make_uint3(bx, by, bz);
        for (unsigned t = 0; t < nt; ++t) {
          getcontext(&f[t].ctx);
          f[t].ctx.uc_stack.ss_sp = &stacks[(size_t)t * kStack];
          f[t].ctx.uc_stack.ss_size = kStack;
          f[t].ctx.uc_link = &g_sched;
          makecontext(&f[t].ctx, fibre_entry, 0);
          f[t].done = false;
          f[t].tid = make_uint3(t % block.x, (t / block.x) % block.y, t / (block.x * block.y));
        }
        bool live = true;
        while (live) {
          live = false;
          for (unsigned t = 0; t < nt; ++t) {
            if (f[t].done) continue;
            g_cur = &f[t];
            threadIdx = f[t].tid;
            swapcontext(&g_sched, &f[t].ctx);
            if (!f[t].done) live = true;
          }
        }
        g_cur = nullptr;
      }
}

/* Kernels without __syncthreads run thread after thread. */
void launch_plain(dim3 grid, dim3 block, const std::function<void()>& body) {
  gridDim = grid;
  blockDim = block;
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        blockIdx = make_uint3(bx, by, bz);
        for (unsigned tz = 0; tz < block.z; ++tz)
          for (unsigned ty = 0; ty < block.y; ++ty)
            for (unsigned tx = 0; tx < block.x; ++tx) {
              threadIdx = make_uint3(tx, ty, tz);
              body();
            }
      }
}

/* computeGridSize (System.cu:641-647) */
void grid_size(int n, int block, int& nb, int& nt) {
  nt = n < block ? n : block;
  nb = n % nt != 0 ? n / nt + 1 : n / nt;
}

/* The reference kernels have no tail guard: every launch covers whole blocks
   and reads element `index` unconditionally.  Sizes whose last block is
   partial would read past the caller's arrays, so they are refused. */
bool size_ok(int n) { return n > 0 && (n <= 64 || n % 512 == 0); }

}  // namespace

void emu_syncthreads() {
  if (!g_cur) {
    fprintf(stderr, "ref_emu: __syncthreads outside a fibre launch\n");
    abort();
  }
  swapcontext(&g_cur->ctx, &g_sched);
}

/* ---- the reference's wrappers on host memory -------------------------- */
extern "C" {

int ref_sizeof_params() { return (int)sizeof(SimParams); }

/* setParameters (System.cu:634-637) */
void ref_set_params(const SimParams* p) { memcpy(&par, p, sizeof(SimParams)); }

/* integrate (System.cu:653-667) */
int ref_integrate(float4* oldPos, float4* newPos, float4* oldVel, float4* newVel, int n) {
  if (!size_ok(n)) return 2;
  int nb, nt;
  grid_size(n, 256, nb, nt);
  launch_plain(dim3(nb), dim3(nt), [&] { integrateD(newPos, newVel, oldPos, oldVel); });
  return 0;
}

/* calcHash (System.cu:671-685) */
int ref_calc_hash(float4* pos, uint2* particleHash, int n) {
  if (!size_ok(n)) return 2;
  int nb, nt;
  grid_size(n, 2 * 256, nb, nt);
  launch_plain(dim3(nb), dim3(nt), [&] { calcHashD(pos, particleHash); });
  return 0;
}

/* RadixSort host loop (radixsort_kernel.cu:445-472), with the kernel grid
   constants of radixsort_kernel.cu:13-44: 48 blocks of 64 threads for the
   sum and shuffle, 16 blocks of 192 for the prefix sum. */
int ref_radix_sort(KeyValuePair* pData0, KeyValuePair* pData1, uint elements, uint bits) {
  uint rounded = elements % 3072 == 0 ? elements : elements + (3072 - elements % 3072);
  for (uint shift = 0; shift < bits; shift += 8) {
    launch_sync(dim3(48), dim3(64), [&] { RadixSum(pData0, elements, rounded, shift); });
    launch_sync(dim3(16), dim3(192), [&] { RadixPrefixSum(); });
    launch_sync(dim3(48), dim3(64),
                [&] { RadixAddOffsetsAndShuffle(pData0, pData1, elements, rounded, (int)shift); });
    KeyValuePair* t = pData0;
    pData0 = pData1;
    pData1 = t;
  }
  return 0;
}

/* reorder (System.cu:689-713) */
int ref_reorder(float4* oldPos, float4* oldVel, float4* sortedPos, float4* sortedVel,
                uint2* particleHash, uint* cellStart, uint n, uint numCells) {
  if (!size_ok((int)n)) return 2;
  int nb, nt;
  grid_size((int)n, 256, nb, nt);
  memset(cellStart, 0xff, numCells * sizeof(uint));
  oldPosTex.ptr = oldPos;
  oldPosTex.count = n;
  oldVelTex.ptr = oldVel;
  oldVelTex.count = n;
  launch_sync(dim3(nb), dim3(nt),
              [&] { reorderD(particleHash, cellStart, oldPos, oldVel, sortedPos, sortedVel); });
  oldPosTex = {};
  oldVelTex = {};
  return 0;
}

/* collide (System.cu:717-756): density pass, then force pass.  newVel is
   written in original particle order through particleHash[i].y. */
int ref_collide(float4* sortedPos, float4* sortedVel, float4* newVel, float4* clr,
                float* pressure, float* density, float* dyeColor, uint2* particleHash,
                uint* cellStart, uint n, uint numCells) {
  if (!size_ok((int)n)) return 2;
  oldPosTex = {sortedPos, n};
  pressureTex = {pressure, n};
  oldVelTex = {sortedVel, n};
  densityTex = {density, n};
  dyeColorTex = {dyeColor, n};
  particleHashTex = {particleHash, n};
  cellStartTex = {cellStart, numCells};
  int nb, nt;
  grid_size((int)n, 64, nb, nt);
  launch_plain(dim3(nb), dim3(nt), [&] {
    computeDensityD(clr, sortedPos, pressure, density, particleHash, cellStart);
  });
  launch_plain(dim3(nb), dim3(nt), [&] {
    computeForceD(nullptr, newVel, sortedPos, sortedVel, clr, pressure, density, dyeColor,
                  particleHash, cellStart);
  });
  oldPosTex = {};
  pressureTex = {};
  oldVelTex = {};
  densityTex = {};
  dyeColorTex = {};
  particleHashTex = {};
  cellStartTex = {};
  return 0;
}

}  // extern "C"
