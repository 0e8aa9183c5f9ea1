/* Stand-in for CUDA/GL interop: the emulated reference build maps no buffers. */
#include <cuda_runtime.h>
