/*
 * gpu_prelude.h -- TEST INFRASTRUCTURE ONLY (part of the oracle).
 *
 * Force-included (nvcc -include) ahead of the kernel sections of the
 * reference's System.cu and radixsort_kernel.cu so that nvcc compiles them
 * for sm_103a as they were written, with texture fetches.  CUDA 13 has no
 * texture references, so each `texture<T, 1, mode>` the reference declares
 * (System.cu:21-30) becomes a __device__ record of a pointer and an element
 * count that the harness (ref_gpu.cpp) fills in where the reference's
 * wrappers bind the texture (System.cu:700, 729-732), and tex1Dfetch returns
 * zero outside [0, count): what a 1D fetch from linear memory returns on the
 * GPU.  The reference relies on that for neighbour cells outside the grid
 * (Kernel_Cell.cui:146-148): their hashes wrap to indices far outside
 * cellStart, so a plain load there would read outside the allocation.
 */
#ifndef REF_GPU_PRELUDE_H
#define REF_GPU_PRELUDE_H

#include <cuda_runtime.h>

template <class T, int dim = 1, enum cudaTextureReadMode mode = cudaReadModeElementType>
struct ref_texture {
  const T* ptr;
  long long count;
};

template <class T, int dim, enum cudaTextureReadMode mode>
__device__ __forceinline__ T tex1Dfetch(const ref_texture<T, dim, mode>& t, int x) {
  if (t.ptr == nullptr || x < 0 || (long long)x >= t.count) return T{};
  return t.ptr[x];
}

/* The reference's file-scope `texture<...> name;` declarations become device
   variables the kernels can read. */
#define texture __device__ ref_texture

#endif
