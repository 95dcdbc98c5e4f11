// batch_strip.cu -- the batched compact forms over column strips: one CTA
// per work unit (column tile x z chunk of some solve), run with the strip
// kernel's unit (strip_unit.cuh).  A unit's record (built by the host) gives
// its tile, chunk, solve and memoryless planes; the solve's constants are
// copied to shared memory, its tensor maps are read by TMA from the
// descriptor in device memory.  Units of solves that reached their step count
// exit at once.  The Mur faces and the step counters follow in the batch's
// other launches (step_fused.cu).  A persistent form (CTAs taking units from
// an atomic counter, the ring continuing from unit to unit) ran 1.12-1.21x
// slower on the same work.  No reference counterpart (the reference runs one
// grid per process).
#include "per_device.h"
#include "strip_unit.cuh"

namespace fdtd {
namespace strip {
namespace {

// One CTA per work unit (the grid is the batch's work list, taken by the
// hardware in unit order like the single-solve kernel's grid): the unit's
// record, its solve's constants in shared memory, then the unit.
template <int RY, int W, int S, bool R16, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) batch_strip_kernel(const BatchDesc *__restrict__ descs,
                                                                  const BatchUnit *__restrict__ units)
{
    using G = StripGeo<RY, W, R16>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ StripConsts s_c;
    const StripSmem sm = strip_smem<RY, W, S, R16>(smem_raw);
    const BatchUnit rec = units[blockIdx.x];
    const int n = *rec.counter;
    if (n >= rec.steps_target)  // the solve is done (uniform over the CTA)
        return;
    strip_init_bars<S>(sm);
    const BatchDesc &d = descs[rec.solve];
    const int par = n & 1;
    if (threadIdx.x == 0)
        strip_consts(s_c, d.c[par]);
    strip_load_coef(d.c[par], sm.coef, G::NTH);
    __syncthreads();
    strip_unit<RY, W, S, R16>(s_c, d.smaps[par], rec.zchunk, rec.bx, rec.by, rec.bz, rec.memless, sm, 0u, false);
    if (threadIdx.x == G::STORE_TID)
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
        fn<<<b.total_units, 32 * W, smem(b.max_classes), s>>>(b.descs, b.units);
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
