// batch_strip.cu -- the batched compact forms over column strips: persistent
// CTAs take work units (column tile x z chunk of some solve) from a counter
// and run them with the strip kernel's unit (strip_unit.cuh); the ring
// continues from unit to unit.  The solve's constants come
// from its descriptor (copied to shared memory), its tensor maps are read by
// TMA from the descriptor in device memory.  Units of solves that reached
// their step count are skipped.  The Mur faces and the step counters follow
// in the batch's other launches (step_fused.cu).  No reference counterpart
// (the reference runs one grid per process).
#include "per_device.h"
#include "strip_unit.cuh"

namespace fdtd {
namespace strip {
namespace {

template <int RY, int W, int S, bool R16, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) batch_strip_kernel(const BatchDesc *__restrict__ descs, int nsolves,
                                                             int total_units, int *work_counter,
                                                             const unsigned long long *__restrict__ memless)
{
    using G = StripGeo<RY, W, R16>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ NativeConsts s_c;
    __shared__ int s_unit, s_solve;
    const StripSmem sm = strip_smem<RY, W, S, R16>(smem_raw);
    strip_init_bars<S>(sm);
    const int tid = threadIdx.x;
    int loaded = -1;
    unsigned g = 0;  // planes staged by this CTA so far
    __syncthreads();
    for (;;) {
        if (tid == 0) {
            const int u = atomicAdd(work_counter, 1);
            int lo = 0, hi = nsolves - 1;
            if (u < total_units) {
                while (lo < hi) {  // last solve with unit_begin <= u
                    const int mid = (lo + hi + 1) >> 1;
                    if (descs[mid].unit_begin <= u)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
            }
            s_unit = u;
            s_solve = lo;
        }
        __syncthreads();
        const int u = s_unit, sv = s_solve;
        if (u >= total_units)
            break;
        const BatchDesc &d = descs[sv];
        const int n = *d.c[0].step_counter;
        if (n < d.steps_target) {
            const int par = n & 1;
            {
                const int *src = reinterpret_cast<const int *>(&d.c[par]);
                int *dst = reinterpret_cast<int *>(&s_c);
                for (int i = tid; i < (int)(sizeof(NativeConsts) / 4); i += G::NTH)
                    dst[i] = src[i];
            }
            if (sv != loaded)
                strip_load_coef(d.c[par], sm.coef, G::NTH);
            __syncthreads();
            loaded = sv;
            const int local = u - d.unit_begin;
            const int per_z = d.tiles_x * d.tiles_y;
            const int bz = local / per_z, rem = local % per_z;
            const int by = rem / d.tiles_x, bx = rem % d.tiles_x;
            const unsigned long long ml = memless ? memless[u] : 0ull;
            if (!strip_unit<RY, W, S, R16>(s_c, d.smaps[par], d.zchunk, bx, by, bz, ml, sm, g, false))
                return;
            g += (unsigned)strip_unit_planes(s_c.nz, d.zchunk, bz);
        }
        __syncthreads();
    }
    if (tid == G::STORE_TID)
        bulk_wait_all();
}

template <int SHAPE, bool R16>
struct BatchKernel {
    static constexpr int RY = Shape<SHAPE>::RY, W = Shape<SHAPE>::W;
    static constexpr int MINB = R16 ? Shape<SHAPE>::BATCH_CTAS16 : Shape<SHAPE>::BATCH_CTAS32;
    static constexpr auto fn = batch_strip_kernel<RY, W, S_SEL, R16, MINB>;
    static int smem(int nclasses) { return strip_smem_bytes<RY, W, S_SEL, R16>(nclasses); }
    // the shared-memory opt-in holds for the current device only
    static int opt_in()
    {
        static PerDeviceOnce<> once;
        int dev = 0;
        const cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess)
            return (int)e;
        const int so = once.run(dev, [] {
            return (int)cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem(FDTD_MAX_CLASSES));
        });
        return so < 0 ? FDTD_ERR_INVALID : so;
    }
    static int ctas(int nclasses)
    {
        if (opt_in() != FDTD_OK)
            return 0;
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * W, smem(nclasses));
        return sms * (per_sm > 0 ? per_sm : 1);
    }
    static int launch(const BatchLaunch &b, cudaStream_t s)
    {
        const int st = opt_in();
        if (st != FDTD_OK)
            return st;
        fn<<<b.persistent_ctas, 32 * W, smem(b.max_classes), s>>>(b.descs, b.nsolves, b.total_units, b.work_counter,
                                                                  b.memless);
        const cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? FDTD_OK : (int)e;
    }
};

template <bool R16>
int launch_shape(const BatchLaunch &b, cudaStream_t s)
{
    switch (b.strip_shape) {
    case 0: return BatchKernel<0, R16>::launch(b, s);
    case 1: return BatchKernel<1, R16>::launch(b, s);
    case 2: return BatchKernel<2, R16>::launch(b, s);
    case 3: return BatchKernel<3, R16>::launch(b, s);
    default: return FDTD_ERR_INVALID;
    }
}

template <bool R16>
int ctas_shape(int shape, int nclasses)
{
    switch (shape) {
    case 0: return BatchKernel<0, R16>::ctas(nclasses);
    case 1: return BatchKernel<1, R16>::ctas(nclasses);
    case 2: return BatchKernel<2, R16>::ctas(nclasses);
    case 3: return BatchKernel<3, R16>::ctas(nclasses);
    default: return 0;
    }
}

}  // namespace
}  // namespace strip

int launch_batch_strip(const BatchLaunch &b, cudaStream_t s)
{
    if (b.max_classes < 1 || b.max_classes > FDTD_MAX_CLASSES)
        return FDTD_ERR_INVALID;
    return b.r16 ? strip::launch_shape<true>(b, s) : strip::launch_shape<false>(b, s);
}

int batch_strip_ctas(bool r16, int shape, int nclasses)
{
    return r16 ? strip::ctas_shape<true>(shape, nclasses) : strip::ctas_shape<false>(shape, nclasses);
}

}  // namespace fdtd
