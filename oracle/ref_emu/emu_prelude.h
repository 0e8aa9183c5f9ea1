/*
 * emu_prelude.h -- TEST INFRASTRUCTURE ONLY (part of the oracle).
 *
 * Force-included (g++ -include) ahead of the reference's own CUDA sources so
 * that g++ compiles their device code for the host CPU.  Nothing in the
 * product links or loads what this builds; it exists to run the reference's
 * kernels here, on a machine with no GPU, and pin the oracle against them.
 *
 * What it provides:
 *   - CUDA qualifiers as no-ops (`__shared__` becomes EMU_SHARED_QUAL, set per
 *     translation unit: `static` for function-scope shared arrays, empty for
 *     the radix sort's `extern __shared__` dynamic array);
 *   - threadIdx/blockIdx/blockDim/gridDim as host globals that the fibre
 *     scheduler in ref_harness.cpp updates before resuming each CUDA thread;
 *   - __syncthreads() as a fibre switch back to that scheduler;
 *   - __mul24 with the hardware's 24-bit signed operand semantics;
 *   - texture references (the reference's USE_TEX build, Params.cuh:5-14):
 *     `texture<T,1,mode>` holds a bound pointer and element count, and
 *     tex1Dfetch returns zero outside [0, count), which is what a 1D fetch
 *     from linear memory returns on the GPU.  The reference relies on that for
 *     neighbour cells outside the grid (Kernel_Cell.cui:146-148).
 *   - float overloads of min/max (the device library has them; the host-side
 *     fallbacks in cutil_math.h only cover int).
 */
#ifndef EMU_PRELUDE_H
#define EMU_PRELUDE_H

#define __device__
#define __host__
#define __global__
#define __constant__
#define __noinline__
#define __forceinline__ inline
#ifndef EMU_SHARED_QUAL
#define EMU_SHARED_QUAL
#endif
#define __shared__ EMU_SHARED_QUAL

#include <cuda_runtime.h>
#include <math.h>
#include <cmath>
#include <stdlib.h>
#include <string.h>

extern uint3 threadIdx;
extern uint3 blockIdx;
extern dim3 blockDim;
extern dim3 gridDim;

void emu_syncthreads();
#define __syncthreads() emu_syncthreads()

static inline int __mul24(int a, int b) {
  int sa = (int)((unsigned)a << 8) >> 8;
  int sb = (int)((unsigned)b << 8) >> 8;
  return (int)(unsigned)((long long)sa * (long long)sb);
}

/* fminf/fmaxf semantics (a NaN operand yields the other one), written out so
   that the host-side fminf/fmaxf stand-ins in cutil_math.h are not involved. */
static inline float min(float a, float b) { return (a < b || b != b) ? a : b; }
static inline float max(float a, float b) { return (a > b || b != b) ? a : b; }
static inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
static inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }

template <class T, int dim = 1, enum cudaTextureReadMode mode = cudaReadModeElementType>
struct texture {
  const T* ptr = nullptr;
  long long count = 0;
};

template <class T, int dim, enum cudaTextureReadMode mode>
static inline T tex1Dfetch(const texture<T, dim, mode>& t, int x) {
  if (t.ptr == nullptr || x < 0 || (long long)x >= t.count) {
    T zero;
    memset(&zero, 0, sizeof(T));
    return zero;
  }
  return t.ptr[x];
}

#endif
