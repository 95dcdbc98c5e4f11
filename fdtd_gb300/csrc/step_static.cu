// step_static.cu -- fdtd_step_static: one single-pass step that allocates no
// device memory.
//
// Who needs it: callers that must not call cudaMalloc -- a host process whose
// device memory is owned by another allocator (a framework's caching pool, a
// fixed budget carved out at start-up), code running where allocation is
// forbidden or would stall other work.  fdtd_plan_create allocates device
// memory for the per-class Debye table, the source table and two status
// words; this entry point keeps those in a file-scope __device__ array
// instead, and takes everything else (fields, classes, Mur slabs) from the
// caller's device buffers.
//
// The array below is a host-side stand-in in host code; its device address is
// looked up with cudaGetSymbolAddress once per device, with that device
// current, on the first call made on it -- so that first call should come
// before any stream capture.  Every GPU that loads the library holds the
// array until the process exits.  All calls share it and it keeps the last
// call's contents: each call rewrites the class table and the source sample
// and clears the error word, so calls whose work overlaps on the GPU race.
#include <algorithm>
#include <mutex>

#include "native.cuh"

namespace fdtd {
namespace {

// Layout: class table (FDTD_STATIC_MAX_CLASSES x 32 B), source sample, error word.
constexpr size_t STATIC_COEF_BYTES = FDTD_STATIC_MAX_CLASSES * sizeof(DebyeCoef);
constexpr size_t STATIC_SCRATCH_BYTES = STATIC_COEF_BYTES + 256;
static_assert(STATIC_SCRATCH_BYTES == FDTD_STATIC_SCRATCH_BYTES, "header and layout disagree");

static __device__ __align__(256) unsigned char g_static_scratch[STATIC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
unsigned char *g_scratch_dev[MAX_DEVICES] = {};

// Device address of the array on the current device (looked up once per device).
int scratch_address(unsigned char **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= MAX_DEVICES)
        return FDTD_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_dev[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_static_scratch);
        if (e != cudaSuccess)
            return e;
        g_scratch_dev[dev] = static_cast<unsigned char *>(ptr);
    }
    *out = g_scratch_dev[dev];
    return FDTD_OK;
}

}  // namespace
}  // namespace fdtd

using namespace fdtd;

extern "C" int fdtd_step_static(const FdtdParams *p, const float *specs, int nclasses, int scheme,
                                const fdtd_native_fields *f, const float *const rp_dev[6], int n,
                                fdtd_stream_t stream)
{
    if (!p || !specs || !f || !rp_dev || n < 0 || p->nx < 3 || p->ny < 3 || p->nz < 3 || p->nz > 65535 ||
        (scheme != FDTD_SCHEME_REFERENCE && scheme != FDTD_SCHEME_CORRECTED))
        return FDTD_ERR_INVALID;
    if (nclasses < 1 || nclasses > FDTD_STATIC_MAX_CLASSES)
        return FDTD_ERR_INVALID;  // the class table must fit the static array
    if (p->sourcesCount < 0 || p->sourcesCount > FDTD_MAX_SOURCES || (p->sourcesCount > 0 && !p->sources))
        return FDTD_ERR_INVALID;
    // the source sample comes from the caller's jz table (this call builds no
    // table): with sources, a table must be given
    if (p->sourcesCount > 0 && (!p->jz || p->jzCount < 1))
        return FDTD_ERR_INVALID;
    for (int s = 0; s < p->sourcesCount; s++) {
        const int *q = p->sources + 3 * s;
        if (q[0] < 1 || q[0] >= p->nx || q[1] < 1 || q[1] >= p->ny || q[2] < 0 || q[2] >= p->nz)
            return FDTD_ERR_INVALID;
    }
    const float *const *fp = &f->hx;
    for (int k = 0; k < 18; k++)
        if (!fp[k])
            return FDTD_ERR_INVALID;
    for (int k = 0; k < 3; k++)
        if ((&f->hx)[k] == (&f->hx_out)[k])
            return FDTD_ERR_INVALID;
    if (!f->material)
        return FDTD_ERR_INVALID;
    for (int k = 0; k < 6; k++)
        if (!rp_dev[k])
            return FDTD_ERR_INVALID;

    unsigned char *scratch = nullptr;
    int st = scratch_address(&scratch);
    if (st != FDTD_OK)
        return st;
    DebyeCoef *d_coef = reinterpret_cast<DebyeCoef *>(scratch);
    float *d_jz = reinterpret_cast<float *>(scratch + STATIC_COEF_BYTES);
    int *d_err = reinterpret_cast<int *>(scratch + STATIC_COEF_BYTES + 4);

    // host-side values: the class table and this step's source sample
    DebyeCoef coef[FDTD_STATIC_MAX_CLASSES];
    for (int k = 0; k < nclasses; k++)
        coef[k] = debye_coef(p->dt, p->eps0, specs[4 * k], specs[4 * k + 1], specs[4 * k + 2], specs[4 * k + 3], scheme);
    // the sample of step n, from the first FDTD_JZ_LEN entries of the table
    // as fdtd_plan_create keeps them (beyond them the sample is 0)
    const int j = scheme == FDTD_SCHEME_CORRECTED ? n : n - n % 3;
    const int njz = p->jz ? std::min(p->jzCount, FDTD_JZ_LEN) : 0;
    const float jz = j < njz ? p->jz[j] : 0.0f;
    struct {
        float jz;
        int err;
    } words = {jz, 0};

    cudaError_t e = cudaMemcpyAsync(d_coef, coef, sizeof(DebyeCoef) * nclasses, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_jz, &words, sizeof words, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess)
        return e;

    NativeConsts c{};
    c.nx = p->nx; c.ny = p->ny; c.nz = p->nz;
    c.pitch = p->nx;
    c.kx = p->dt / (p->mu0 * p->dx);
    c.ky = p->dt / (p->mu0 * p->dy);
    c.kz = p->dt / (p->mu0 * p->dz);
    c.tx = p->dt / p->dx;
    c.ty = p->dt / p->dy;
    c.tz = p->dt / p->dz;
    c.dt = p->dt;
    c.hx = p->dx; c.hy = p->dy; c.hz = p->dz;
    c.me = p->mu0 * p->eps0;
    c.scheme = scheme;
    c.nsources = p->sourcesCount;
    for (int k = 0; k < 3 * p->sourcesCount; k++)
        c.sources[k] = p->sources[k];
    c.coef = d_coef;
    c.nclasses = nclasses;
    c.jz = d_jz;          // one entry: the sample of step n, selected above
    c.njz = 1;
    c.step = 0;
    c.step_counter = nullptr;
    c.err = d_err;
    c.stall_once = nullptr;
    c.rp = MurSlabs{rp_dev[0], rp_dev[1], rp_dev[2], rp_dev[3], rp_dev[4], rp_dev[5]};
    for (int k = 0; k < 3; k++) {
        c.h_in[k] = (&f->hx)[k];
        c.h_out[k] = (&f->hx_out)[k];
        c.e_cur[k] = (&f->ex)[k];
        c.e_prev[k] = (&f->ex_prev)[k];
        c.d_cur[k] = (&f->dx)[k];
        c.d_prev[k] = (&f->dx_prev)[k];
    }
    c.mat = f->material;

    st = launch_h_de_fused(c, stream);
    if (st == FDTD_OK)
        st = launch_mur(c, stream);
    if (st != FDTD_OK)
        return st;
    // read the error word behind the step on the caller's stream, wait for
    // both, and report a bounded wait that gave up
    int err = 0;
    e = cudaMemcpyAsync(&err, d_err, sizeof err, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess)
        return e;
    return err ? FDTD_ERR_DEVICE_TIMEOUT : FDTD_OK;
}
