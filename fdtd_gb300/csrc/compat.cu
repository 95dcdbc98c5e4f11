// compat.cu -- reference-compatible launchers (fdtd_calculations.h:18-42).
//
// Same argument lists and per-component index ranges as the reference's five
// kernels, over the reference's float material arrays and three-slot state.
// The grids differ: 32 x 8 thread tiles instead of 128 x 1 rows, sources as
// one warp instead of a full grid, Mur over the face cells only.
#include <array>
#include <atomic>

#include "device_common.cuh"

namespace fdtd {
namespace {

// The reference's __constant__ block (fdtd_calculations.h:10-15).
struct SymbolBlock {
    int nx, ny, nz;
    float dt, dx, dy, dz, mu0, eps0;
    int nsources;
    int sources[3 * FDTD_MAX_SOURCES];
    int njz;
};

__constant__ SymbolBlock c_sym;
// The whole source table; the reference's dJz holds 512 entries.
__device__ float g_jz[FDTD_JZ_LEN];

std::array<std::atomic<bool>, 128> g_symbols_ready{};
std::array<SymbolBlock, 128> g_host_sym{};

int current_device_checked(int *dev)
{
    cudaError_t e = cudaGetDevice(dev);
    if (e != cudaSuccess)
        return e;
    if (*dev < 0 || *dev >= (int)g_symbols_ready.size())
        return FDTD_ERR_INVALID;
    return FDTD_OK;
}

int launch_status()
{
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FDTD_OK : (int)e;
}

constexpr int TX = 32, TY = 8;

__global__ void __launch_bounds__(TX *TY) compat_h_kernel(float *__restrict__ hx, float *__restrict__ hy,
                                                         float *__restrict__ hz, const float *__restrict__ ex,
                                                         const float *__restrict__ ey, const float *__restrict__ ez)
{
    const int nx = c_sym.nx, ny = c_sym.ny, nz = c_sym.nz;
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y, z = blockIdx.z;
    if (x >= nx || y >= ny)
        return;
    const float dt = c_sym.dt, mu0 = c_sym.mu0;
    const float kx = dt / (mu0 * c_sym.dx), ky = dt / (mu0 * c_sym.dy), kz = dt / (mu0 * c_sym.dz);
    const size_t i = cell_index(x, y, z, nx, ny);
    const size_t sx = 1, sy = nx, sz = (size_t)nx * ny;
    // hx: x 1..nx-2, y 0..ny-2, z 0..nz-2; both terms scaled by dy (:48-52)
    if (x >= 1 && x < nx - 1 && y < ny - 1 && z < nz - 1)
        hx[i] = hx[i] - ky * (ez[i + sy] - ez[i]) + ky * (ey[i + sz] - ey[i]);
    // hy: x 0..nx-2, y 1..ny-2, z 0..nz-2 (:60-64)
    if (x < nx - 1 && y >= 1 && y < ny - 1 && z < nz - 1)
        hy[i] = hy[i] - kz * (ex[i + sz] - ex[i]) + kx * (ez[i + sx] - ez[i]);
    // hz: x 0..nx-2, y 0..ny-2, z 1..nz-2 (:71-75)
    if (x < nx - 1 && y < ny - 1 && z >= 1 && z < nz - 1)
        hz[i] = hz[i] - kx * (ey[i + sx] - ey[i]) + ky * (ex[i + sy] - ex[i]);
}

__global__ void __launch_bounds__(TX *TY) compat_d_kernel(float *__restrict__ dxT, float *__restrict__ dyT,
                                                         float *__restrict__ dzT, const float *__restrict__ dxS,
                                                         const float *__restrict__ dyS, const float *__restrict__ dzS,
                                                         const float *__restrict__ hx, const float *__restrict__ hy,
                                                         const float *__restrict__ hz)
{
    const int nx = c_sym.nx, ny = c_sym.ny, nz = c_sym.nz;
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y, z = blockIdx.z;
    if (x >= nx || y >= ny)
        return;
    const float tx = c_sym.dt / c_sym.dx, ty = c_sym.dt / c_sym.dy, tz = c_sym.dt / c_sym.dz;
    const size_t i = cell_index(x, y, z, nx, ny);
    const size_t sx = 1, sy = nx, sz = (size_t)nx * ny;
    if (x < nx - 1 && y >= 1 && y < ny - 1 && z >= 1 && z < nz - 1)
        dxT[i] = dxS[i] + ty * (hz[i] - hz[i - sy]) - tz * (hy[i] - hy[i - sz]);
    if (x >= 1 && x < nx - 1 && y < ny - 1 && z >= 1 && z < nz - 1)
        dyT[i] = dyS[i] + tz * (hx[i] - hx[i - sz]) - tx * (hz[i] - hz[i - sx]);
    if (x >= 1 && x < nx - 1 && y >= 1 && y < ny - 1 && z < nz - 1)
        dzT[i] = dzS[i] + tx * (hy[i] - hy[i - sx]) - ty * (hx[i] - hx[i - sy]);
}

struct ETriplet {
    float *t[3];
    const float *e0[3], *e1[3], *d0[3], *d1[3], *d2[3];
};

__global__ void __launch_bounds__(TX *TY) compat_e_kernel(ETriplet a, const float *__restrict__ sigma,
                                                         const float *__restrict__ eps_i,
                                                         const float *__restrict__ eps_s,
                                                         const float *__restrict__ tau_d)
{
    const int nx = c_sym.nx, ny = c_sym.ny, nz = c_sym.nz;
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y, z = blockIdx.z;
    if (x >= nx || y >= ny)
        return;
    // ex: x 0..nx-2, y 1..ny-2, z 1..nz-2; ey, ez: x 1..nx-1, y 0..ny-1, z 1..nz-1 (:147-175)
    const bool ex_on = x < nx - 1 && y >= 1 && y < ny - 1 && z >= 1 && z < nz - 1;
    const bool eyz_on = x >= 1 && z >= 1;
    if (!ex_on && !eyz_on)
        return;
    const size_t i = cell_index(x, y, z, nx, ny);
    const DebyeCoef k = cell_coef(c_sym.dt, c_sym.eps0, sigma[i], eps_s[i], eps_i[i], tau_d[i], FDTD_SCHEME_REFERENCE);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (c == 0 ? !ex_on : !eyz_on)
            continue;
        a.t[c][i] = debye_update(k, a.e0[c][i], a.e1[c][i], a.d0[c][i], a.d1[c][i], a.d2[c][i]);
    }
}

__global__ void compat_sources_kernel(float *__restrict__ dzT, const float *__restrict__ dzS,
                                      const float *__restrict__ hx, const float *__restrict__ hy, int iter)
{
    const int s = threadIdx.x;
    if (s >= c_sym.nsources)
        return;
    const int nx = c_sym.nx, ny = c_sym.ny;
    const int x = c_sym.sources[3 * s], y = c_sym.sources[3 * s + 1], z = c_sym.sources[3 * s + 2];
    const size_t i = cell_index(x, y, z, nx, ny);
    const float jz = (iter >= 0 && iter < c_sym.njz) ? g_jz[iter] : 0.0f;
    dzT[i] = dzS[i] + c_sym.dt / c_sym.dx * (hy[i] - hy[i - 1]) - c_sym.dt / c_sym.dy * (hx[i] - hx[i - nx]) - jz;
}

struct MurArgs {
    float *t[3];
    const float *s[3];
    MurSlabs rp;
};

__global__ void __launch_bounds__(256) compat_mur_kernel(MurArgs a)
{
    const int nx = c_sym.nx, ny = c_sym.ny, nz = c_sym.nz;
    const int f = blockIdx.y;
    const MurFace m = mur_face(f, nx, ny, nz);
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)m.len_u * m.len_v)
        return;
    const int iu = (int)(idx % m.len_u), iv = (int)(idx / m.len_u);
    mur_apply(f, iu, iv, nx, ny, nz, nx, c_sym.dt, c_sym.dx, c_sym.dy, c_sym.dz, c_sym.mu0 * c_sym.eps0, a.rp, a.t[0],
              a.t[1], a.t[2], a.s[0], a.s[1], a.s[2], false);
}

int prologue(SymbolBlock *sym)
{
    int dev;
    int st = current_device_checked(&dev);
    if (st != FDTD_OK)
        return st;
    if (!g_symbols_ready[dev].load())
        return FDTD_ERR_NO_SYMBOLS;
    *sym = g_host_sym[dev];
    return FDTD_OK;
}

dim3 cell_grid(const SymbolBlock &s) { return dim3((s.nx + TX - 1) / TX, (s.ny + TY - 1) / TY, s.nz); }

}  // namespace
}  // namespace fdtd

using namespace fdtd;

extern "C" {

int fdtd_copy_symbols(const FdtdParams *p)
{
    if (!p || p->nx < 3 || p->ny < 3 || p->nz < 3 || p->sourcesCount < 0 || p->sourcesCount > FDTD_MAX_SOURCES ||
        (p->sourcesCount > 0 && !p->sources) || p->jzCount < 0 || (p->jzCount > 0 && !p->jz))
        return FDTD_ERR_INVALID;
    if ((long long)p->nx * p->ny * p->nz > (1LL << 40) || p->nz > 65535)
        return FDTD_ERR_INVALID;
    for (int s = 0; s < p->sourcesCount; s++) {
        const int *q = p->sources + 3 * s;
        // updateSources reads hy at x-1 and hx at y-1 (:206-207).
        if (q[0] < 1 || q[0] >= p->nx || q[1] < 1 || q[1] >= p->ny || q[2] < 0 || q[2] >= p->nz)
            return FDTD_ERR_INVALID;
    }
    int dev;
    int st = current_device_checked(&dev);
    if (st != FDTD_OK)
        return st;
    SymbolBlock s{};
    s.nx = p->nx; s.ny = p->ny; s.nz = p->nz;
    s.dt = p->dt; s.dx = p->dx; s.dy = p->dy; s.dz = p->dz;
    s.mu0 = p->mu0; s.eps0 = p->eps0;
    s.nsources = p->sourcesCount;
    for (int k = 0; k < 3 * p->sourcesCount; k++)
        s.sources[k] = p->sources[k];
    s.njz = p->jzCount < FDTD_JZ_LEN ? p->jzCount : FDTD_JZ_LEN;
    cudaError_t e = cudaMemcpyToSymbol(c_sym, &s, sizeof s);
    if (e == cudaSuccess && s.njz > 0)
        e = cudaMemcpyToSymbol(g_jz, p->jz, sizeof(float) * s.njz);
    if (e != cudaSuccess)
        return e;
    g_host_sym[dev] = s;
    g_symbols_ready[dev].store(true);
    return FDTD_OK;
}

int fdtd_update_h(float *hx, float *hy, float *hz, const float *exSource, const float *eySource,
                  const float *ezSource, fdtd_stream_t stream)
{
    SymbolBlock s;
    int st = prologue(&s);
    if (st != FDTD_OK)
        return st;
    if (!hx || !hy || !hz || !exSource || !eySource || !ezSource)
        return FDTD_ERR_INVALID;
    compat_h_kernel<<<cell_grid(s), dim3(TX, TY), 0, stream>>>(hx, hy, hz, exSource, eySource, ezSource);
    return launch_status();
}

int fdtd_update_d(float *dxTarget, float *dyTarget, float *dzTarget, const float *dxSource, const float *dySource,
                  const float *dzSource, const float *hx, const float *hy, const float *hz, fdtd_stream_t stream)
{
    SymbolBlock s;
    int st = prologue(&s);
    if (st != FDTD_OK)
        return st;
    if (!dxTarget || !dyTarget || !dzTarget || !dxSource || !dySource || !dzSource || !hx || !hy || !hz)
        return FDTD_ERR_INVALID;
    compat_d_kernel<<<cell_grid(s), dim3(TX, TY), 0, stream>>>(dxTarget, dyTarget, dzTarget, dxSource, dySource,
                                                              dzSource, hx, hy, hz);
    return launch_status();
}

int fdtd_update_e(float *exTarget, float *eyTarget, float *ezTarget, const float *exSource0, const float *eySource0,
                  const float *ezSource0, const float *exSource1, const float *eySource1, const float *ezSource1,
                  const float *dxSource0, const float *dySource0, const float *dzSource0, const float *dxSource1,
                  const float *dySource1, const float *dzSource1, const float *dxSource2, const float *dySource2,
                  const float *dzSource2, const float *sigma, const float *epsI, const float *epsS, const float *tauD,
                  fdtd_stream_t stream)
{
    SymbolBlock s;
    int st = prologue(&s);
    if (st != FDTD_OK)
        return st;
    ETriplet a{{exTarget, eyTarget, ezTarget},
               {exSource0, eySource0, ezSource0},
               {exSource1, eySource1, ezSource1},
               {dxSource0, dySource0, dzSource0},
               {dxSource1, dySource1, dzSource1},
               {dxSource2, dySource2, dzSource2}};
    for (int c = 0; c < 3; c++)
        if (!a.t[c] || !a.e0[c] || !a.e1[c] || !a.d0[c] || !a.d1[c] || !a.d2[c])
            return FDTD_ERR_INVALID;
    if (!sigma || !epsI || !epsS || !tauD)
        return FDTD_ERR_INVALID;
    compat_e_kernel<<<cell_grid(s), dim3(TX, TY), 0, stream>>>(a, sigma, epsI, epsS, tauD);
    return launch_status();
}

int fdtd_update_sources(float *dzTarget, const float *dzSource, const float *hx, const float *hy, int currIteration,
                        fdtd_stream_t stream)
{
    SymbolBlock s;
    int st = prologue(&s);
    if (st != FDTD_OK)
        return st;
    if (!dzTarget || !dzSource || !hx || !hy)
        return FDTD_ERR_INVALID;
    if (s.nsources == 0)
        return FDTD_OK;
    compat_sources_kernel<<<1, 32, 0, stream>>>(dzTarget, dzSource, hx, hy, currIteration);
    return launch_status();
}

int fdtd_update_mur(float *exTarget, float *eyTarget, float *ezTarget, const float *exSource, const float *eySource,
                    const float *ezSource, const float *rpx0, const float *rpy0, const float *rpz0,
                    const float *rpxEnd, const float *rpyEnd, const float *rpzEnd, fdtd_stream_t stream)
{
    SymbolBlock s;
    int st = prologue(&s);
    if (st != FDTD_OK)
        return st;
    MurArgs a{{exTarget, eyTarget, ezTarget}, {exSource, eySource, ezSource}, {rpx0, rpy0, rpz0, rpxEnd, rpyEnd, rpzEnd}};
    for (int c = 0; c < 3; c++)
        if (!a.t[c] || !a.s[c])
            return FDTD_ERR_INVALID;
    if (!rpx0 || !rpy0 || !rpz0 || !rpxEnd || !rpyEnd || !rpzEnd)
        return FDTD_ERR_INVALID;
    long long most = 0;
    for (int f = 0; f < 12; f++) {
        const MurFace m = mur_face(f, s.nx, s.ny, s.nz);
        most = std::max(most, (long long)m.len_u * m.len_v);
    }
    compat_mur_kernel<<<dim3((unsigned)((most + 255) / 256), 12), 256, 0, stream>>>(a);
    return launch_status();
}

}  // extern "C"
