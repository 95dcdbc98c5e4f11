/*
 * ref_cpu.cpp -- runs the reference's own kernel bodies on the CPU.
 *
 * Test infrastructure only.  Built by oracle/build.py in a container that
 * holds the reference sources: the reference kernel file is compiled as C++
 * with ref_shim_cpu.h force-included, and this harness loops each kernel over
 * the reference's launch grid (ceil(nx/128) x ny x nz blocks of 128 x 1 x 1,
 * fdtd.cu:13-15,75-78) with the reference's slot rotation (fdtd.cu:115-530).
 * Its outputs pin the oracle restatement bit for bit.
 *
 * Threads with ix >= nx are skipped: in every reference kernel they write
 * nothing; updateEField would only read its per-cell coefficients past the
 * end of the arrays (fdtd_calculations.cu:141-144) and discard them.
 */
#include "fdtd_calculations.cu"

#include <omp.h>

namespace {

int g_nx, g_ny, g_nz;

template <class K>
void launch(K kernel)
{
    const int bxs = (g_nx + 127) / 128;
    #pragma omp parallel for schedule(static)
    for (int bz = 0; bz < g_nz; bz++) {
        blockDim = {128, 1, 1};
        for (int by = 0; by < g_ny; by++)
            for (int bx = 0; bx < bxs; bx++) {
                blockIdx = {bx, by, bz};
                for (int tx = 0; tx < 128 && bx * 128 + tx < g_nx; tx++) {
                    threadIdx = {tx, 0, 0};
                    kernel();
                }
            }
    }
}

}  // namespace

extern "C" {

int ref_cpu_set_symbols(int nx, int ny, int nz, float dt, float dx, float dy, float dz, float mu0,
                        float eps0, int nsources, const int *sources, const float *jz, int njz)
{
    FdtdParams p;
    memset(&p, 0, sizeof p);
    p.nx = nx; p.ny = ny; p.nz = nz;
    p.dt = dt; p.dx = dx; p.dy = dy; p.dz = dz;
    p.mu0 = mu0; p.eps0 = eps0;
    p.sourcesCount = nsources;
    p.sources = const_cast<int *>(sources);
    p.jzCount = njz;
    p.jz = const_cast<float *>(jz);
    copySymbolsToDevice(&p);
    g_nx = nx; g_ny = ny; g_nz = nz;
    return 0;
}

void ref_cpu_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }

int ref_cpu_update_h(float **h, float **e)
{
    launch([&] { updateHField(h[0], h[1], h[2], e[0], e[1], e[2]); });
    return 0;
}

int ref_cpu_update_d(float **dT, float **dS, float **h)
{
    launch([&] { updateDField(dT[0], dT[1], dT[2], dS[0], dS[1], dS[2], h[0], h[1], h[2]); });
    return 0;
}

int ref_cpu_update_sources(float *dzT, float *dzS, float *hx, float *hy, int iter)
{
    blockDim = {128, 1, 1};
    blockIdx = {0, 0, 0};
    threadIdx = {0, 0, 0};
    updateSources(dzT, dzS, hx, hy, iter);
    return 0;
}

/* media: sigma, epsI, epsS, tauD */
int ref_cpu_update_e(float **eT, float **e0, float **e1, float **d0, float **d1, float **d2, float **m)
{
    launch([&] {
        updateEField(eT[0], eT[1], eT[2], e0[0], e0[1], e0[2], e1[0], e1[1], e1[2],
                     d0[0], d0[1], d0[2], d1[0], d1[1], d1[2], d2[0], d2[1], d2[2],
                     m[0], m[1], m[2], m[3]);
    });
    return 0;
}

/* rp: rpx0, rpy0, rpz0, rpxEnd, rpyEnd, rpzEnd */
int ref_cpu_update_mur(float **eT, float **eS, float **rp)
{
    launch([&] {
        updateMurBoundary(eT[0], eT[1], eT[2], eS[0], eS[1], eS[2], rp[0], rp[1], rp[2], rp[3], rp[4], rp[5]);
    });
    return 0;
}

/* state: hx hy hz, e slot0 xyz, e slot1 xyz, e slot2 xyz, d slot0 xyz, d slot1 xyz, d slot2 xyz */
int ref_cpu_run(float **state, float **media, float **rp, int step0, int nsteps)
{
    float **h = state;
    float **e[3] = {state + 3, state + 6, state + 9};
    float **d[3] = {state + 12, state + 15, state + 18};
    for (int i = step0; i < step0 + nsteps; i++) {
        const int t = i % 3, n0 = (i + 2) % 3, n1 = (i + 1) % 3;
        ref_cpu_update_h(h, e[n0]);
        ref_cpu_update_d(d[t], d[n0], h);
        ref_cpu_update_sources(d[t][2], d[n0][2], h[0], h[1], i - i % 3);
        ref_cpu_update_e(e[t], e[n0], e[n1], d[t], d[n0], d[n1], media);
        ref_cpu_update_mur(e[t], e[n0], rp);
    }
    return 0;
}

}  // extern "C"
