// native.cu -- the native fused path: plan, H kernel, D+source+E kernel, Mur.
//
// State (fdtd_native_fields): H, two E slots, two D slots, a uint8 material
// class per cell.  Step n reads E^n, D^n from the current slots and E^{n-1},
// D^{n-1} from the "prev" slots, which receive E^{n+1}, D^{n+1} cell by cell
// after they are read.  Every cell is either written on every step or never
// written, so two slots reproduce the reference's three-slot rotation
// (fdtd.cu:115-530) exactly.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "device_common.cuh"
#include "native.cuh"
#include "fdtd_internal.h"

namespace fdtd {

DebyeCoef debye_coef(float dt, float eps0, float sigma, float eps_s, float eps_i, float tau, int scheme)
{
    // updateEField's per-cell coefficients (fdtd_calculations.cu:141-144),
    // double literals and float storage exactly as there.
    DebyeCoef k{};
    const float a = 2.0 * eps0 * eps_i * tau;
    const float b = a + 2.0 * dt * (eps0 * eps_s + sigma * tau);
    const float c = 1.0 / (b + sigma * dt * dt);
    const float d = scheme == FDTD_SCHEME_CORRECTED ? (1.0 * a + b - sigma * dt * dt) : (2.0 * b - sigma * dt * dt);
    k.a = a;
    k.c = c;
    k.d = d;
    k.two_dt = 2.0f * dt;
    k.two_tau = 2.0f * tau;
    const float s = dt + tau;
    k.delta = (float)(2.0 * ((double)s - ((double)dt + (double)tau)));
    return k;
}

int scan_material(const uint8_t *mat, int nx, int ny, int nz, int nclasses, unsigned long long *hash, int *top_class)
{
    // Per z plane, in parallel: the largest class, and a fingerprint made of
    // four FNV-1a chains over the plane's little-endian 64-bit words (word i
    // feeds chain i % 4, so the four multiplies overlap), its tail bytes fed
    // to chain 0.  The chains, then the plane fingerprints, are folded in
    // order by FNV-1a over their bytes.
    constexpr unsigned long long FNV_BASIS = 1469598103934665603ULL, FNV_PRIME = 1099511628211ULL;
    auto fold = [](unsigned long long h, unsigned long long v) {
        for (int b = 0; b < 8; b++)
            h = (h ^ ((v >> (8 * b)) & 0xffu)) * FNV_PRIME;
        return h;
    };
    const size_t plane = (size_t)nx * ny;
    std::vector<unsigned long long> ph(nz);
    std::vector<int> top(nz, 0);
    parallel_for(nz, 0, [&](int z) {
        const uint8_t *q = mat + (size_t)z * plane;
        unsigned long long lane[4] = {FNV_BASIS, FNV_BASIS ^ 1, FNV_BASIS ^ 2, FNV_BASIS ^ 3};
        const size_t quads = plane / 32;
        for (size_t i = 0; i < quads; i++) {
            unsigned long long w[4];
            std::memcpy(w, q + 32 * i, sizeof w);
            for (int l = 0; l < 4; l++) {
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_BIG_ENDIAN__
                w[l] = __builtin_bswap64(w[l]);  // little-endian words on every host
#endif
                lane[l] = (lane[l] ^ w[l]) * FNV_PRIME;
            }
        }
        for (size_t i = 32 * quads; i < plane; i++)
            lane[0] = (lane[0] ^ q[i]) * FNV_PRIME;
        unsigned long long h = FNV_BASIS;
        for (int l = 0; l < 4; l++)
            h = fold(h, lane[l]);
        ph[z] = h;
        uint8_t m = 0;  // a max reduction the compiler vectorises
        for (size_t i = 0; i < plane; i++)
            m = q[i] > m ? q[i] : m;
        top[z] = m;
    });
    unsigned long long h = FNV_BASIS;
    int m = 0;
    for (int z = 0; z < nz; z++) {
        if (top[z] >= nclasses)
            return FDTD_ERR_INVALID;
        m = std::max(m, top[z]);
        h = fold(h, ph[z]);
    }
    if (hash)
        *hash = h;
    if (top_class)
        *top_class = m;
    return FDTD_OK;
}

NativeConsts make_consts(const fdtd_plan *p, const fdtd_native_fields *f, int n)
{
    NativeConsts c{};
    c.nx = p->nx;
    c.ny = p->ny;
    c.nz = p->nz;
    c.pitch = p->nx;
    c.kx = p->dt / (p->mu0 * p->dx);
    c.ky = p->dt / (p->mu0 * p->dy);
    c.kz = p->dt / (p->mu0 * p->dz);
    c.tx = p->dt / p->dx;
    c.ty = p->dt / p->dy;
    c.tz = p->dt / p->dz;
    c.dt = p->dt;
    c.hx = p->dx;
    c.hy = p->dy;
    c.hz = p->dz;
    c.me = p->mu0 * p->eps0;
    c.scheme = p->scheme;
    c.nsources = p->nsources;
    for (int s = 0; s < p->nsources; s++)
        for (int k = 0; k < 3; k++)
            c.sources[3 * s + k] = p->sources[3 * s + k];
    c.coef = p->d_coef;
    c.nclasses = p->nclasses;
    c.jz = p->d_jz;
    c.njz = p->njz;
    c.rp = p->rp;
    c.mur_x = p->d_mur_x;
    for (int k = 0; k < 6; k++)
        for (int j = 0; j < 4; j++)
            c.mur_k[k][j] = p->mur_k[k][j];
    c.mur_uniform = p->mur_uniform;
    c.step = n;
    c.step_counter = nullptr;
    c.err = p->d_err;
    c.stall_once = p->d_stall;
    if (f) {
        for (int k = 0; k < 3; k++) {
            c.h_in[k] = (&f->hx)[k];
            c.h_out[k] = (&f->hx_out)[k];
            c.e_cur[k] = (&f->ex)[k];
            c.e_prev[k] = (&f->ex_prev)[k];
            c.d_cur[k] = (&f->dx)[k];
            c.d_prev[k] = (&f->dx_prev)[k];
        }
        c.mat = f->material;
    }
    return c;
}

namespace {

constexpr int TX = 32, TY = 8;

__device__ __forceinline__ DebyeCoef load_coef(const DebyeCoef *__restrict__ table, int cls)
{
    const float4 *p = reinterpret_cast<const float4 *>(table + cls);
    const float4 u = __ldg(p), v = __ldg(p + 1);
    DebyeCoef k;
    k.a = u.x; k.c = u.y; k.d = u.z; k.two_dt = u.w;
    k.two_tau = v.x; k.delta = v.y; k.pad0 = v.z; k.pad1 = v.w;
    return k;
}

// updateHField (fdtd_calculations.cu:32-77) with separate in and out buffers
// (they may alias).
__global__ void __launch_bounds__(TX *TY) native_h_kernel(NativeConsts c)
{
    const int nx = c.nx, ny = c.ny, nz = c.nz;
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y, z = blockIdx.z;
    if (x >= nx - 1 || y >= ny - 1 || z >= nz - 1)
        return;  // no H component is updated at x = nx-1, y = ny-1 or z = nz-1
    const size_t i = cell_index(x, y, z, nx, ny);
    const size_t sx = 1, sy = nx, sz = (size_t)nx * ny;
    const float *__restrict__ ex = c.e_cur[0];
    const float *__restrict__ ey = c.e_cur[1];
    const float *__restrict__ ez = c.e_cur[2];
    const float ex0 = ex[i], ey0 = ey[i], ez0 = ez[i];
    if (x >= 1)
        c.h_out[0][i] = c.h_in[0][i] - c.ky * (ez[i + sy] - ez0) + c.ky * (ey[i + sz] - ey0);
    if (y >= 1)
        c.h_out[1][i] = c.h_in[1][i] - c.kz * (ex[i + sz] - ex0) + c.kx * (ez[i + sx] - ez0);
    if (z >= 1)
        c.h_out[2][i] = c.h_in[2][i] - c.kx * (ey[i + sx] - ey0) + c.ky * (ex[i + sy] - ex0);
}

__device__ __forceinline__ int source_sample_index(const NativeConsts &c, int n)
{
    return c.scheme == FDTD_SCHEME_CORRECTED ? n : n - n % 3;
}

// updateDField + updateSources + updateEField for one cell (fdtd_calculations.cu
// :80-122, :187-213, :125-184).  H^{n+1/2} is read from h_out.
__global__ void __launch_bounds__(TX *TY) native_de_kernel(NativeConsts c)
{
    const int nx = c.nx, ny = c.ny, nz = c.nz;
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y, z = blockIdx.z;
    if (x >= nx || y >= ny)
        return;
    const size_t i = cell_index(x, y, z, nx, ny);
    const size_t sx = 1, sy = nx, sz = (size_t)nx * ny;
    const float *__restrict__ hx = c.h_out[0];
    const float *__restrict__ hy = c.h_out[1];
    const float *__restrict__ hz = c.h_out[2];

    const bool xi = x >= 1 && x < nx - 1, yi = y >= 1 && y < ny - 1, zi = z >= 1 && z < nz - 1;
    const bool dx_on = x < nx - 1 && yi && zi;
    const bool dy_on = xi && y < ny - 1 && zi;
    bool dz_on = xi && yi && z < nz - 1;
    const bool ex_on = x < nx - 1 && yi && zi;
    const bool eyz_on = x >= 1 && z >= 1;

    // soft source at this cell? (block-uniform screen first)
    bool is_src = false;
    if (c.nsources > 0) {
        const int bx0 = blockIdx.x * TX, by0 = blockIdx.y * TY;
        for (int s = 0; s < c.nsources; s++) {
            const int sx_ = c.sources[3 * s], sy_ = c.sources[3 * s + 1], sz_ = c.sources[3 * s + 2];
            if (sz_ == z && sx_ >= bx0 && sx_ < bx0 + TX && sy_ >= by0 && sy_ < by0 + TY)
                is_src |= (sx_ == x && sy_ == y);
        }
    }
    if (!ex_on && !eyz_on && !dx_on && !dy_on && !dz_on && !is_src)
        return;

    float dn[3], dp[3], dnew[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        dn[k] = c.d_cur[k][i];
        dp[k] = c.d_prev[k][i];
        dnew[k] = dp[k];  // untouched cells keep the slot's value
    }
    if (dx_on)
        dnew[0] = dn[0] + c.ty * (hz[i] - hz[i - sy]) - c.tz * (hy[i] - hy[i - sz]);
    if (dy_on)
        dnew[1] = dn[1] + c.tz * (hx[i] - hx[i - sz]) - c.tx * (hz[i] - hz[i - sx]);
    if (dz_on || is_src) {
        dnew[2] = dn[2] + c.tx * (hy[i] - hy[i - sx]) - c.ty * (hx[i] - hx[i - sy]);
        if (is_src) {
            const int n = c.step_counter ? *c.step_counter : c.step;
            const int j = source_sample_index(c, n);
            dnew[2] = dnew[2] - ((j >= 0 && j < c.njz) ? c.jz[j] : 0.0f);
        }
        dz_on = true;
    }
    if (dx_on) c.d_prev[0][i] = dnew[0];
    if (dy_on) c.d_prev[1][i] = dnew[1];
    if (dz_on) c.d_prev[2][i] = dnew[2];

    if (ex_on || eyz_on) {
        const DebyeCoef k = load_coef(c.coef, c.mat[i]);
#pragma unroll
        for (int m = 0; m < 3; m++) {
            if (m == 0 ? !ex_on : !eyz_on)
                continue;
            const float e0 = c.e_cur[m][i], e1 = c.e_prev[m][i];
            c.e_prev[m][i] = debye_update(k, e0, e1, dnew[m], dn[m], dp[m]);
        }
    }
}

// updateMurBoundary over the face cells of the native state: blockIdx.z is
// the face set, x runs along its faster in-face axis, y (strided) along the
// other.  The last block to run cannot be known, so block (0, 0, 0) advances
// the device step counter (no other block of this launch reads it).
constexpr int MUR_THREADS = 128;
constexpr int MUR_ROWS = 4;  // face rows per thread, loads issued together

__global__ void __launch_bounds__(MUR_THREADS) native_mur_kernel(NativeConsts c)
{
    // the next step's single-pass kernel may launch now; its CTAs that read
    // or write what this kernel touches wait for this grid to complete
    asm volatile("griddepcontrol.launch_dependents;");
    const int f = blockIdx.z;
    const MurFace m = mur_face(f, c.nx, c.ny, c.nz);
    if (c.step_counter && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0)
        atomicAdd(c.step_counter, 1);
    const int iu = blockIdx.x * MUR_THREADS + threadIdx.x;
    if (iu >= m.len_u)
        return;
    int len_v = m.len_v;
    if (m.axis == 0 && (mur_x_fused_faces(c) & (m.far ? 2 : 1))) {
        if (m.comp == 1)
            return;  // the single-pass kernel updated this ey face
        len_v = 1;   // ez: only the z = 0 row is left
    }
    const bool fix = c.scheme == FDTD_SCHEME_CORRECTED;
    const int slab = m.axis + 3 * m.far;
    if ((c.mur_uniform >> slab) & 1) {
        // one value in the set's slab: its factors, picked by constant indices
        // (a run-time index into the argument block would copy it to local memory)
        float4 kf = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
        for (int s = 0; s < 6; s++)
            if (s == slab)
                kf = make_float4(c.mur_k[s][0], c.mur_k[s][1], c.mur_k[s][2], c.mur_k[s][3]);
        for (int iv = blockIdx.y; iv < len_v; iv += MUR_ROWS * gridDim.y)
            mur_apply_k<MUR_ROWS, true>(f, iu, iv, gridDim.y, len_v, c.nx, c.ny, c.nz, c.pitch, c.dt, c.hx, c.hy, c.hz,
                                        c.me, c.rp, c.e_prev[0], c.e_prev[1], c.e_prev[2], c.e_cur[0], c.e_cur[1],
                                        c.e_cur[2], fix, kf);
        return;
    }
    for (int iv = blockIdx.y; iv < len_v; iv += MUR_ROWS * gridDim.y)
        mur_apply_k<MUR_ROWS>(f, iu, iv, gridDim.y, len_v, c.nx, c.ny, c.nz, c.pitch, c.dt, c.hx, c.hy, c.hz, c.me, c.rp,
                              c.e_prev[0], c.e_prev[1], c.e_prev[2], c.e_cur[0], c.e_cur[1], c.e_cur[2], fix);
}

int launch_status()
{
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FDTD_OK : (int)e;
}

// n copies of v from dst on (slabs and face factors that hold one value).
template <class T>
__global__ void __launch_bounds__(256) fill_kernel(T *__restrict__ dst, size_t n, T v)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = v;
}

template <class T>
cudaError_t fill_on(T *dst, size_t n, T v, cudaStream_t stream)
{
    if (n == 0)
        return cudaSuccess;
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 1024);
    fill_kernel<T><<<blocks, 256, 0, stream>>>(dst, n, v);
    return cudaGetLastError();
}

bool fields_ok(const fdtd_native_fields *f, bool need_h_out)
{
    if (!f)
        return false;
    const float *const *ptrs = &f->hx;
    for (int k = 0; k < 18; k++)
        if (!ptrs[k] && (need_h_out || k < 3 || k >= 6))
            return false;
    return f->material != nullptr;
}

}  // namespace

int launch_h(const NativeConsts &c, cudaStream_t s)
{
    const dim3 grid((c.nx + TX - 1) / TX, (c.ny + TY - 1) / TY, c.nz);
    native_h_kernel<<<grid, dim3(TX, TY), 0, s>>>(c);
    return launch_status();
}

int launch_de(const NativeConsts &c, cudaStream_t s)
{
    const dim3 grid((c.nx + TX - 1) / TX, (c.ny + TY - 1) / TY, c.nz);
    native_de_kernel<<<grid, dim3(TX, TY), 0, s>>>(c);
    return launch_status();
}

int launch_mur(const NativeConsts &c, cudaStream_t s)
{
    int most_u = 1, most_v = 1;
    for (int f = 0; f < 12; f++) {
        const MurFace m = mur_face(f, c.nx, c.ny, c.nz);
        most_u = std::max(most_u, m.len_u);
        most_v = std::max(most_v, m.len_v);
    }
    const int rows = (most_v + MUR_ROWS - 1) / MUR_ROWS;
    const dim3 grid((unsigned)((most_u + MUR_THREADS - 1) / MUR_THREADS), (unsigned)std::min(rows, 65535), 12);
    native_mur_kernel<<<grid, MUR_THREADS, 0, s>>>(c);
    return launch_status();
}

int plan_error(const fdtd_plan *p)
{
    int flag = 0;
    cudaError_t e = cudaMemcpy(&flag, p->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return e;
    if (flag) {
        cudaMemset(p->d_err, 0, sizeof(int));
        return FDTD_ERR_DEVICE_TIMEOUT;
    }
    return FDTD_OK;
}

}  // namespace fdtd

using namespace fdtd;

extern "C" {

int fdtd_plan_create(const FdtdParams *p, const float *specs, int nclasses, int scheme,
                     const float *const rp_host[6], fdtd_plan **out)
{
    return plan_create_on(p, specs, nclasses, scheme, rp_host, nullptr, nullptr, out);
}

}  // extern "C"

namespace fdtd {

int plan_params_check(const FdtdParams *p, int scheme)
{
    if (!p || p->nx < 3 || p->ny < 3 || p->nz < 3 || p->nz > 65535 || p->sourcesCount < 0 ||
        p->sourcesCount > FDTD_MAX_SOURCES || (scheme != FDTD_SCHEME_REFERENCE && scheme != FDTD_SCHEME_CORRECTED))
        return FDTD_ERR_INVALID;
    for (int s = 0; s < p->sourcesCount; s++) {
        const int *q = p->sources + 3 * s;
        if (q[0] < 1 || q[0] >= p->nx || q[1] < 1 || q[1] >= p->ny || q[2] < 0 || q[2] >= p->nz)
            return FDTD_ERR_INVALID;
    }
    return FDTD_OK;
}

int plan_create_on(const FdtdParams *p, const float *specs, int nclasses, int scheme, const float *const rp_host[6],
                   cudaMemPool_t pool, cudaStream_t stream, fdtd_plan **out)
{
    if (!specs || !out || nclasses < 1 || nclasses > FDTD_MAX_CLASSES || plan_params_check(p, scheme) != FDTD_OK)
        return FDTD_ERR_INVALID;
    fdtd_plan *plan = new (std::nothrow) fdtd_plan();
    if (!plan)
        return FDTD_ERR_NOMEM;
    plan->nx = p->nx; plan->ny = p->ny; plan->nz = p->nz;
    plan->dt = p->dt; plan->dx = p->dx; plan->dy = p->dy; plan->dz = p->dz;
    plan->mu0 = p->mu0; plan->eps0 = p->eps0;
    plan->scheme = scheme;
    plan->nclasses = nclasses;
    plan->nsources = p->sourcesCount;
    for (int k = 0; k < 3 * p->sourcesCount; k++)
        plan->sources[k] = p->sources[k];

    // Debye coefficient table per class; all 256 entries exist so that any
    // uint8 class index reads inside the table (unused entries are zero)
    std::vector<DebyeCoef> coef(FDTD_MAX_CLASSES, DebyeCoef{});
    for (int k = 0; k < nclasses; k++)
        coef[k] = debye_coef(p->dt, p->eps0, specs[4 * k], specs[4 * k + 1], specs[4 * k + 2], specs[4 * k + 3], scheme);
    plan->host_coef = coef;

    // source table
    std::vector<float> jz(FDTD_JZ_LEN, 0.0f);
    if (p->jz && p->jzCount > 0) {
        std::copy(p->jz, p->jz + std::min(p->jzCount, FDTD_JZ_LEN), jz.begin());
    } else {
        FdtdParams q = *p;
        q.jz = nullptr;
        q.jzCount = 0;
        const int st = fdtd_setup_sources(&q);
        if (st != FDTD_OK) {
            delete plan;
            return st;
        }
        std::copy(q.jz, q.jz + FDTD_JZ_LEN, jz.begin());
        std::free(q.jz);
    }
    plan->njz = FDTD_JZ_LEN;

    // Mur slabs (from the default material when not given, as the reference
    // computes them before loadMaterials, fdtd.cu:59,65).  A slab whose
    // entries are all one value (every slab made from the default material)
    // is filled on the device and never built on the host.
    const size_t nrp[6] = {2 * (size_t)p->ny * p->nz, (size_t)p->nx * 2 * p->nz, (size_t)p->nx * p->ny * 2,
                           2 * (size_t)p->ny * p->nz, (size_t)p->nx * 2 * p->nz, (size_t)p->nx * p->ny * 2};
    float one_value[6] = {};
    bool one[6] = {};
    if (rp_host) {
        for (int k = 0; k < 6; k++) {
            if (!rp_host[k]) {
                delete plan;
                return FDTD_ERR_INVALID;
            }
            // one value: every entry with the first one's bits (and not a NaN)
            const float v = rp_host[k][0];
            uint32_t vb;
            std::memcpy(&vb, &v, sizeof vb);
            one[k] = v == v;
            for (size_t i = 0; i < nrp[k] && one[k]; i++) {
                uint32_t b;
                std::memcpy(&b, rp_host[k] + i, sizeof b);
                one[k] = b == vb;
            }
            one_value[k] = v;
        }
    } else {
        // fdtd_setup_mur_uniform's two values: x slabs, y and z slabs
        const float vx = mur_rp_value(p, p->defaultSigma, p->defaultEpsS, p->defaultEpsI, p->defaultTauD, false);
        const float vyz = mur_rp_value(p, p->defaultSigma, p->defaultEpsS, p->defaultEpsI, p->defaultTauD, true);
        for (int k = 0; k < 6; k++) {
            one[k] = true;
            one_value[k] = k % 3 == 0 ? vx : vyz;
        }
    }

    // one-valued slabs: their factors once, rounded one operation at a time
    // as mur_value rounds them (IEEE single, no contraction)
    {
        const float me = p->mu0 * p->eps0, dt = p->dt;
        const float hs[3] = {p->dx, p->dy, p->dz};
        for (int k = 0; k < 6; k++) {
            if (!one[k])
                continue;
            const float q = hs[k % 3] * std::sqrt(me * one_value[k]);
            plan->mur_k[k][0] = 1.0f / (dt + q);
            plan->mur_k[k][1] = dt - q;
            plan->mur_k[k][2] = dt + q;
            plan->mur_k[k][3] = dt - q;
            plan->mur_uniform |= 1 << k;
        }
    }

    size_t total = 0;
    size_t offs[8];
    offs[0] = 0;
    offs[1] = (sizeof(DebyeCoef) * FDTD_MAX_CLASSES + 255) & ~size_t(255);
    size_t cur = offs[1] + ((sizeof(float) * FDTD_JZ_LEN + 255) & ~size_t(255));
    for (int k = 0; k < 6; k++) {
        offs[2 + k] = cur;
        cur += (sizeof(float) * nrp[k] + 255) & ~size_t(255);
    }
    const size_t murx_off = cur;
    const size_t nmurx = 2 * (size_t)p->nz * p->ny;
    cur += (sizeof(float4) * nmurx + 255) & ~size_t(255);
    const size_t err_off = cur;
    total = cur + 256;
    char *base = nullptr;
    cudaError_t e = pool ? cudaMallocFromPoolAsync(reinterpret_cast<void **>(&base), total, pool, stream)
                         : cudaMalloc(&base, total);
    if (e != cudaSuccess) {
        delete plan;
        return e;
    }
    plan->d_block = base;
    plan->pooled = pool != nullptr;
    // Copies and fills are ordered on `stream` (null: the legacy default
    // stream), which is synchronised before the host vectors below go away.
    auto put = [&](void *dst, const void *src, size_t n) {
        return cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, stream);
    };
    plan->d_coef = reinterpret_cast<DebyeCoef *>(base + offs[0]);
    plan->d_jz = reinterpret_cast<float *>(base + offs[1]);
    float *rpd[6];
    for (int k = 0; k < 6; k++)
        rpd[k] = reinterpret_cast<float *>(base + offs[2 + k]);
    plan->rp = MurSlabs{rpd[0], rpd[1], rpd[2], rpd[3], rpd[4], rpd[5]};
    plan->d_err = reinterpret_cast<int *>(base + err_off);
    plan->d_stall = plan->d_err + 1;
    plan->d_mur_x = reinterpret_cast<float4 *>(base + murx_off);
    std::vector<float4> murx;
    {
        // The x-face Mur factors of mur_value, rounded one operation at a time
        // in the same order (IEEE single: sqrt and division correctly rounded,
        // no contraction), so the kernel that applies them gets the bits the
        // Mur kernel gets from the slabs.  A one-valued x slab gives one
        // factor set for its whole face (its mur_k row).
        const float me = p->mu0 * p->eps0, dt = p->dt, h = p->dx;
        const size_t per_face = (size_t)p->nz * p->ny;
        for (int face = 0; face < 2 && e == cudaSuccess; face++) {
            const int k = face ? 3 : 0;
            float4 *dst = plan->d_mur_x + face * per_face;
            if (one[k]) {
                e = fill_on(dst, per_face, make_float4(plan->mur_k[k][0], plan->mur_k[k][1], plan->mur_k[k][2],
                                                       plan->mur_k[k][3]), stream);
                continue;
            }
            if (murx.empty())
                murx.resize(nmurx);
            const float *slab = rp_host[k];
            float last_self = 0.0f, last_nbr = 0.0f;
            float4 v{};
            bool have = false;  // v holds the factors of (last_self, last_nbr)
            for (int z = 0; z < p->nz; z++)
                for (int y = 0; y < p->ny; y++) {
                    const size_t b = ((size_t)z * p->ny + y) * 2;
                    const float r_self = slab[b + (face ? 1 : 0)], r_nbr = slab[b + (face ? 0 : 1)];
                    if (!have || r_self != last_self || r_nbr != last_nbr) {
                        const float q_self = h * std::sqrt(me * r_self), q_nbr = h * std::sqrt(me * r_nbr);
                        v.x = 1.0f / (dt + q_self);
                        v.y = dt - q_nbr;
                        v.z = dt + q_nbr;
                        v.w = dt - q_self;
                        last_self = r_self;
                        last_nbr = r_nbr;
                        have = true;
                    }
                    murx[(size_t)face * per_face + (size_t)z * p->ny + y] = v;
                }
            e = put(dst, murx.data() + face * per_face, sizeof(float4) * per_face);
        }
        if (e == cudaSuccess)  // error flag, test hook word
            e = cudaMemsetAsync(plan->d_err, 0, 2 * sizeof(int), stream);
        if (e == cudaSuccess)
            e = put(plan->d_coef, coef.data(), sizeof(DebyeCoef) * FDTD_MAX_CLASSES);
        if (e == cudaSuccess)
            e = put(plan->d_jz, jz.data(), sizeof(float) * FDTD_JZ_LEN);
        for (int k = 0; k < 6 && e == cudaSuccess; k++)
            e = one[k] ? fill_on(rpd[k], nrp[k], one_value[k], stream)
                       : put(rpd[k], rp_host[k], sizeof(float) * nrp[k]);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(stream);  // the host vectors are released below
    }
    if (e != cudaSuccess) {
        if (pool)
            cudaFreeAsync(base, stream);
        else
            cudaFree(base);
        delete plan;
        return e;
    }
    cudaGetDevice(&plan->device);
    *out = plan;
    return FDTD_OK;
}

void plan_destroy_on(fdtd_plan *plan, cudaStream_t stream)
{
    if (!plan)
        return;
    if (plan->pooled)
        cudaFreeAsync(plan->d_block, stream);
    else
        cudaFree(plan->d_block);
    delete plan;
}

}  // namespace fdtd

extern "C" {

int fdtd_plan_status(fdtd_plan *plan)
{
    if (!plan)
        return FDTD_ERR_INVALID;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
        return e;
    return plan_error(plan);
}

int fdtd_plan_destroy(fdtd_plan *plan)
{
    if (!plan)
        return FDTD_OK;
    cudaError_t e = plan->pooled ? cudaFreeAsync(plan->d_block, nullptr) : cudaFree(plan->d_block);
    delete plan;
    return e == cudaSuccess ? FDTD_OK : (int)e;
}

int fdtd_step_h(const fdtd_plan *plan, const fdtd_native_fields *f, fdtd_stream_t stream)
{
    if (!plan || !fields_ok(f, true))
        return FDTD_ERR_INVALID;
    return launch_h(make_consts(plan, f, 0), stream);
}

int fdtd_step_de(const fdtd_plan *plan, const fdtd_native_fields *f, int n, fdtd_stream_t stream)
{
    if (!plan || !fields_ok(f, true) || n < 0)
        return FDTD_ERR_INVALID;
    const NativeConsts c = make_consts(plan, f, n);
    int st = launch_de(c, stream);
    if (st == FDTD_OK)
        st = launch_mur(c, stream);
    return st;
}

int fdtd_step(const fdtd_plan *plan, const fdtd_native_fields *f, int n, fdtd_stream_t stream)
{
    if (!plan || !fields_ok(f, true) || n < 0)
        return FDTD_ERR_INVALID;
    for (int k = 0; k < 3; k++)
        if ((&f->hx)[k] == (&f->hx_out)[k])
            return FDTD_ERR_INVALID;
    return launch_step(make_consts(plan, f, n), stream);
}

}  // extern "C"
