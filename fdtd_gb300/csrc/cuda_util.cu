// cuda_util.cu -- CUDA error text for status codes below FDTD_ERR_INVALID.
#include <cuda_runtime.h>

#include "fdtd_internal.h"

namespace fdtd {

const char *cuda_error_string(int code)
{
    if (code > 0 && code < FDTD_ERR_INVALID)
        return cudaGetErrorString(static_cast<cudaError_t>(code));
    return "unknown status";
}

}  // namespace fdtd
