/*
 * ref_gpu.cu -- runs the reference's own CUDA kernels on the GPU.
 *
 * Test and measurement infrastructure only.  The reference kernel file
 * (fdtd_calculations.cu) is compiled, unchanged and with the reference
 * Makefile's default nvcc options plus the sm_103a target, into a cubin by
 * oracle/build.py where the reference sources exist; this harness (our own
 * code, built on any host) loads that cubin with the driver API, fills the
 * kernels' __constant__ block the way copySymbolsToDevice does
 * (fdtd_calculations.cu:7-29), and drives the five kernels with the
 * reference's launch configuration (grid ceil(nx/128) x ny x nz, blocks of
 * 128 x 1 x 1; fdtd.cu:13-15,75-78) and slot rotation (fdtd.cu:115-530) on one
 * stream, with snapshot output gated off.
 *
 * Guards against the reference's unchecked accesses:
 *  - updateEField reads its per-cell coefficients before the bounds check
 *    (fdtd_calculations.cu:141-144), so threads with ix >= nx read up to 127
 *    floats past the end of the material arrays when nx % 128 != 0: every
 *    array here is allocated with 128 floats of zero padding.
 *  - updateSources reads dJz[i - i % 3] from a 512-entry constant array
 *    (fdtd_calculations.cu:208, fdtd.cu:172): runs are refused unless every
 *    step index stays below 512.
 *  - sources at x = 0 or y = 0 would read before hy / hx, and more than 16
 *    would read past dSources: refused.
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

namespace {

CUmodule g_mod = nullptr;
CUfunction g_fn[5] = {};  // H, D, sources, E, Mur
const char *const FN_NAMES[5] = {"updateHField", "updateDField", "updateSources", "updateEField",
                                 "updateMurBoundary"};

int cu(CUresult r) { return r == CUDA_SUCCESS ? 0 : (int)r; }
int rt(cudaError_t e) { return e == cudaSuccess ? 0 : 20000 + (int)e; }

int set_symbol(const char *name, const void *src, size_t bytes)
{
    CUdeviceptr p = 0;
    size_t size = 0;
    int st = cu(cuModuleGetGlobal(&p, &size, g_mod, name));
    if (st)
        return st;
    if (bytes > size)
        return 30001;
    return cu(cuMemcpyHtoD(p, src, bytes));
}

}  // namespace

extern "C" {

typedef struct RefGpuProblem {
    int nx, ny, nz;
    float dt, dx, dy, dz, mu0, eps0;
    int nsources;
    const int *sources;           /* 3 per source, 0-based x, y, z */
    int njz;
    const float *jz;
    const float *media[4];        /* host, nx*ny*nz each: sigma, epsI, epsS, tauD */
    const float *rp[6];           /* host: rpx0, rpy0, rpz0, rpxEnd, rpyEnd, rpzEnd */
} RefGpuProblem;

/* Loads the reference kernels; returns 0 or an error code. */
int ref_gpu_load(const char *cubin_path)
{
    if (g_mod)
        return 0;
    int st = rt(cudaFree(nullptr));  // primary context current on this thread
    if (st)
        return st;
    st = cu(cuModuleLoad(&g_mod, cubin_path));
    if (st)
        return st;
    unsigned count = 0;
    st = cu(cuModuleGetFunctionCount(&count, g_mod));
    if (st)
        return st;
    std::vector<CUfunction> fns(count);
    st = cu(cuModuleEnumerateFunctions(fns.data(), count, g_mod));
    if (st)
        return st;
    for (CUfunction f : fns) {
        const char *name = nullptr;
        if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name)
            continue;
        for (int k = 0; k < 5; k++)
            if (std::strstr(name, FN_NAMES[k]))
                g_fn[k] = f;
    }
    for (int k = 0; k < 5; k++)
        if (!g_fn[k])
            return 30002;
    return 0;
}

/*
 * Runs warmup + nsteps steps from a zero state.  state_out (optional) receives
 * 21 arrays of nx*ny*nz floats: hx hy hz, E slot 0 xyz, E slot 1 xyz, E slot 2
 * xyz, D slot 0 xyz, D slot 1 xyz, D slot 2 xyz.  ms_out (optional) receives
 * the CUDA-event time of the nsteps timed steps.
 */
int ref_gpu_run(const RefGpuProblem *p, int warmup, int nsteps, float *state_out, float *ms_out)
{
    if (!g_mod || !p || p->nx < 3 || p->ny < 3 || p->nz < 3 || warmup < 0 || nsteps < 0)
        return 30003;
    const int last = warmup + nsteps - 1;
    if (last >= 0 && last - last % 3 >= 512)
        return 30004;
    if (p->nsources < 0 || p->nsources > 16)
        return 30005;
    for (int s = 0; s < p->nsources; s++) {
        const int x = p->sources[3 * s], y = p->sources[3 * s + 1], z = p->sources[3 * s + 2];
        if (x < 1 || x >= p->nx || y < 1 || y >= p->ny || z < 0 || z >= p->nz)
            return 30005;
    }
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const size_t n = (size_t)nx * ny * nz;
    const size_t padded = (n + 128) * sizeof(float);
    const size_t rpn[6] = {2 * (size_t)ny * nz, (size_t)nx * 2 * nz, (size_t)nx * ny * 2,
                           2 * (size_t)ny * nz, (size_t)nx * 2 * nz, (size_t)nx * ny * 2};

    // constant block (copySymbolsToDevice)
    int st = 0;
    st = st ? st : set_symbol("dNx", &p->nx, sizeof(int));
    st = st ? st : set_symbol("dNy", &p->ny, sizeof(int));
    st = st ? st : set_symbol("dNz", &p->nz, sizeof(int));
    st = st ? st : set_symbol("dDt", &p->dt, sizeof(float));
    st = st ? st : set_symbol("dDx", &p->dx, sizeof(float));
    st = st ? st : set_symbol("dDy", &p->dy, sizeof(float));
    st = st ? st : set_symbol("dDz", &p->dz, sizeof(float));
    st = st ? st : set_symbol("dMu0", &p->mu0, sizeof(float));
    st = st ? st : set_symbol("dEps0", &p->eps0, sizeof(float));
    st = st ? st : set_symbol("dSourcesCount", &p->nsources, sizeof(int));
    if (p->nsources > 0)
        st = st ? st : set_symbol("dSources", p->sources, sizeof(int) * 3 * p->nsources);
    {
        float jz[512] = {};
        const int njz = p->njz < 512 ? p->njz : 512;
        if (njz > 0)
            std::memcpy(jz, p->jz, sizeof(float) * njz);
        st = st ? st : set_symbol("dJz", jz, sizeof jz);
    }
    if (st)
        return st;

    // device arrays: 21 state + 4 media + 6 rp, zero padded
    std::vector<float *> bufs;
    auto alloc = [&](size_t bytes) -> float * {
        void *q = nullptr;
        if (cudaMalloc(&q, bytes) != cudaSuccess)
            return nullptr;
        bufs.push_back(static_cast<float *>(q));
        if (cudaMemset(q, 0, bytes) != cudaSuccess)
            return nullptr;
        return static_cast<float *>(q);
    };
    float *state[21], *media[4], *rp[6];
    bool ok = true;
    for (int k = 0; k < 21 && ok; k++)
        ok = (state[k] = alloc(padded)) != nullptr;
    for (int k = 0; k < 4 && ok; k++)
        ok = (media[k] = alloc(padded)) != nullptr &&
             cudaMemcpy(media[k], p->media[k], n * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    for (int k = 0; k < 6 && ok; k++)
        ok = (rp[k] = alloc((rpn[k] + 128) * sizeof(float))) != nullptr &&
             cudaMemcpy(rp[k], p->rp[k], rpn[k] * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (ok)
        ok = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreate(&ev0) == cudaSuccess && cudaEventCreate(&ev1) == cudaSuccess;
    if (!ok)
        st = 30006;

    float **h = state;
    float **e[3] = {state + 3, state + 6, state + 9};
    float **d[3] = {state + 12, state + 15, state + 18};
    const unsigned gx = (unsigned)((nx + 127) / 128);
    auto launch = [&](int k, std::vector<void *> args) {
        return cu(cuLaunchKernel(g_fn[k], gx, (unsigned)ny, (unsigned)nz, 128, 1, 1, 0, (CUstream)stream,
                                 args.data(), nullptr));
    };
    auto step = [&](int i) {
        const int t = i % 3, n0 = (i + 2) % 3, n1 = (i + 1) % 3;
        int iter = i - i % 3;
        int r = launch(0, {&h[0], &h[1], &h[2], &e[n0][0], &e[n0][1], &e[n0][2]});
        r = r ? r
              : launch(1, {&d[t][0], &d[t][1], &d[t][2], &d[n0][0], &d[n0][1], &d[n0][2], &h[0], &h[1], &h[2]});
        r = r ? r : launch(2, {&d[t][2], &d[n0][2], &h[0], &h[1], &iter});
        r = r ? r
              : launch(3, {&e[t][0], &e[t][1], &e[t][2], &e[n0][0], &e[n0][1], &e[n0][2], &e[n1][0], &e[n1][1],
                           &e[n1][2], &d[t][0], &d[t][1], &d[t][2], &d[n0][0], &d[n0][1], &d[n0][2], &d[n1][0],
                           &d[n1][1], &d[n1][2], &media[0], &media[1], &media[2], &media[3]});
        r = r ? r
              : launch(4, {&e[t][0], &e[t][1], &e[t][2], &e[n0][0], &e[n0][1], &e[n0][2], &rp[0], &rp[1], &rp[2],
                           &rp[3], &rp[4], &rp[5]});
        return r;
    };
    for (int i = 0; i < warmup && !st; i++)
        st = step(i);
    if (!st)
        st = rt(cudaEventRecord(ev0, stream));
    for (int i = warmup; i < warmup + nsteps && !st; i++)
        st = step(i);
    if (!st)
        st = rt(cudaEventRecord(ev1, stream));
    if (!st)
        st = rt(cudaStreamSynchronize(stream));
    if (!st && ms_out)
        st = rt(cudaEventElapsedTime(ms_out, ev0, ev1));
    for (int k = 0; k < 21 && !st && state_out; k++)
        st = rt(cudaMemcpy(state_out + (size_t)k * n, state[k], n * sizeof(float), cudaMemcpyDeviceToHost));
    if (ev0)
        cudaEventDestroy(ev0);
    if (ev1)
        cudaEventDestroy(ev1);
    if (stream)
        cudaStreamDestroy(stream);
    for (float *b : bufs)
        cudaFree(b);
    return st;
}

}  // extern "C"
