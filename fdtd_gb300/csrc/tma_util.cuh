// tma_util.cuh -- helpers shared by the z-marching kernels: mbarriers with
// bounded waits, TMA tile loads, cp.async copies, tensor-map encoding.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstring>
#include <mutex>

namespace fdtd {
namespace tma {

constexpr int FTX = 32;            // tile width in x (one warp)
constexpr int MBAR_SPIN_LIMIT = 1 << 22;
constexpr unsigned long long MBAR_WAIT_NS = 200000000ull;  // a wait gives up after 0.2 s

__host__ __device__ constexpr int pad128(int bytes) { return (bytes + 127) & ~127; }

// ---------------------------------------------------------------- PTX helpers

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: false after MBAR_SPIN_LIMIT polls or, once 16384 polls
// failed, after MBAR_WAIT_NS of the global timer (read every 256 polls).  The
// first polls read no timer: with the timer read after the first failed poll
// both step kernels ran 0.7-1.1 % slower.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    constexpr int FAST_POLLS = 16384;
    for (int i = 0; i < FAST_POLLS; i++)
        if (mbar_try_wait(bar, parity))
            return true;
    const unsigned long long t0 = globaltimer_ns();
    for (int i = FAST_POLLS; i < MBAR_SPIN_LIMIT; i++) {
        if (mbar_try_wait(bar, parity))
            return true;
        if ((i & 255) == 0 && globaltimer_ns() - t0 > MBAR_WAIT_NS)
            return false;
    }
    return false;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// 1-D bulk copy global -> shared, completing on an mbarrier (both addresses
// 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void cp_async4(uint32_t dst, const void *src, bool valid)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(valid ? 4 : 0) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// ------------------------------------------------------------ plane staging

enum PlaneKind { PLANE_FULL = 0, PLANE_PRO = 1, PLANE_EPI = 2 };


__device__ __forceinline__ int plane_kind(int z, int zc0, int zc1)
{
    return z < zc0 ? PLANE_PRO : (z >= zc1 ? PLANE_EPI : PLANE_FULL);
}


inline PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// Tensor map of a 3-D array of es-byte elements of type dt: dims (d0, d1,
// d2), element strides s1 between rows and s2 between planes, box (b0, b1, 1).
inline bool encode_map_3d(PFN_cuTensorMapEncodeTiled_v12000 fn, CUtensorMap *m, const void *base,
                          CUtensorMapDataType dt, size_t es, int d0, int d1, int d2, size_t s1, size_t s2, int b0,
                          int b1)
{
    cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)d1, (cuuint64_t)d2};
    cuuint64_t strides[2] = {(cuuint64_t)(s1 * es), (cuuint64_t)(s2 * es)};
    cuuint32_t box[3] = {(cuuint32_t)b0, (cuuint32_t)b1, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(m, dt, 3, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

inline bool encode_map(PFN_cuTensorMapEncodeTiled_v12000 fn, CUtensorMap *m, const void *base, bool is_u8, int nx, int ny,
                int nz, int pitch, int bx, int by)
{
    return encode_map_3d(fn, m, base, is_u8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                         is_u8 ? 1 : 4, nx, ny, nz, (size_t)pitch, (size_t)pitch * ny, bx, by);
}

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace tma
}  // namespace fdtd
