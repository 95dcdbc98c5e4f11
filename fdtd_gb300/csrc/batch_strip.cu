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
__global__ void __launch_bounds__(32 * W, MINB) batch_strip_kernel(const BatchDesc *__restrict__ descs,
                                                                   int total_units, int *work_counter,
                                                                   const BatchUnit *__restrict__ units)
{
    using G = StripGeo<RY, W, R16>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ StripConsts s_c;
    __shared__ BatchUnit s_rec[2];  // the current unit's record and the next one's
    __shared__ int s_unit, s_n;
    const StripSmem sm = strip_smem<RY, W, S, R16>(smem_raw);
    strip_init_bars<S>(sm);
    const int tid = threadIdx.x;
    int loaded = -1;    // solve * 2 + parity whose constants s_c holds
    int coef_of = -1;   // solve whose class table is loaded
    unsigned g = 0;     // planes staged by this CTA so far
    // thread 0 takes units one ahead: `next` is the unit after the current
    // one (its record is copied to shared memory while the current one
    // runs), `ahead` the counter value taken for the unit after that
    int next = 0, ahead = 0;
    auto fetch = [&](int u, int slot) {
        if (u < total_units) {
            cp_async16(smem_addr(&s_rec[slot]), &units[u]);
            cp_async16(smem_addr(&s_rec[slot]) + 16, reinterpret_cast<const unsigned char *>(&units[u]) + 16);
        }
        cp_async_commit();
    };
    if (tid == 0) {
        next = atomicAdd(work_counter, 1);
        fetch(next, 0);
        ahead = atomicAdd(work_counter, 1);
    }
    for (int i = 0;; i++) {
        const int slot = i & 1;
        if (tid == 0) {
            cp_async_wait<0>();
            const int u = next;
            s_unit = u;
            // the solve's completed steps, or -1 once it reached its target
            const int n = u < total_units ? *s_rec[slot].counter : 0;
            s_n = u < total_units && n < s_rec[slot].steps_target ? n : -1;
            if (u < total_units) {
                next = ahead;
                fetch(next, slot ^ 1);  // read by all threads one unit ago, before the barrier below
                ahead = next < total_units ? atomicAdd(work_counter, 1) : total_units;
            }
        }
        __syncthreads();
        const int u = s_unit;
        if (u >= total_units)
            break;
        const BatchUnit rec = s_rec[slot];
        const BatchDesc &d = descs[rec.solve];
        const int n = s_n;
        if (n >= 0) {
            const int par = n & 1;
            const bool consts = rec.solve * 2 + par != loaded, coef = rec.solve != coef_of;
            if (consts && tid == 0)
                strip_consts(s_c, d.c[par]);
            if (coef)
                strip_load_coef(d.c[par], sm.coef, G::NTH);
            if (consts || coef)
                __syncthreads();
            loaded = rec.solve * 2 + par;
            coef_of = rec.solve;
            if (!strip_unit<RY, W, S, R16>(s_c, d.smaps[par], rec.zchunk, rec.bx, rec.by, rec.bz, rec.memless, sm, g,
                                           false)) {
                if (tid == 0)
                    cp_async_wait<0>();
                return;
            }
            g += (unsigned)strip_unit_planes(s_c.nz, rec.zchunk, rec.bz);
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
        fn<<<b.persistent_ctas, 32 * W, smem(b.max_classes), s>>>(b.descs, b.total_units, b.work_counter, b.units);
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
