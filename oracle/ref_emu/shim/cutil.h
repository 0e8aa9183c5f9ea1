/* Stand-in for the CUDA SDK cutil.h: error-check macros are not needed by the device code compiled here. */
#include <cuda_runtime.h>
#define CUDA_SAFE_CALL(x) (x)
#define CUT_CHECK_ERROR(m)
