// cuda_util.cu -- CUDA error text for status codes below FDTD_ERR_INVALID,
// and page-locked host memory for asynchronous copies.
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

extern "C" int fdtd_host_alloc(size_t bytes, void **out)
{
    if (!out || bytes == 0)
        return FDTD_ERR_INVALID;
    *out = nullptr;
    const cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocDefault);
    return e == cudaSuccess ? FDTD_OK : (int)e;
}

extern "C" int fdtd_host_free(void *p)
{
    const cudaError_t e = cudaFreeHost(p);
    return e == cudaSuccess ? FDTD_OK : (int)e;
}
