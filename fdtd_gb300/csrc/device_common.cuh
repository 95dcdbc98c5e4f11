// device_common.cuh -- device helpers shared by the compat and native kernels.
#pragma once

#include <cuda_runtime.h>

#include "fdtd_internal.h"

namespace fdtd {

__host__ __device__ inline size_t cell_index(int x, int y, int z, int nx, int ny)
{
    return ((size_t)z * (size_t)ny + (size_t)y) * (size_t)nx + (size_t)x;
}

// Debye E update of one component (fdtd_calculations.cu:150-156): E^{n+1} =
// c (d E^n - a E^{n-1} + k1 D^{n+1} - k2 D^n + k3 D^{n-1}), the D terms in
// the difference form of DebyeCoef.
__device__ __forceinline__ float debye_update(const DebyeCoef &k, float e0, float e1, float d0, float d1, float d2)
{
    const float p = k.d * e0 - k.a * e1;
    const float g1 = d0 - d1;
    const float g2 = d1 - d2;
    const float q = k.two_dt * g1 + k.two_tau * (g1 - g2) + k.delta * d0;
    return k.c * (p + q);
}

// The reference's per-cell coefficients (fdtd_calculations.cu:141-144) in
// single precision.  The reference evaluates a, b, c, d with double literals;
// here c is the correctly rounded reciprocal of the same float sum, d is the
// same single rounding, a and b may differ from it by one unit in the last
// place.  delta comes from an exact two-sum of dt + tau.
__device__ __forceinline__ DebyeCoef cell_coef(float dt, float eps0, float sigma, float eps_s, float eps_i, float tau,
                                               int scheme)
{
    DebyeCoef k;
    const float a = 2.0f * eps0 * eps_i * tau;
    const float b = a + 2.0f * dt * (eps0 * eps_s + sigma * tau);
    const float s = __fmul_rn(__fmul_rn(sigma, dt), dt);
    k.a = a;
    k.c = __frcp_rn(__fadd_rn(b, s));
    k.d = scheme == FDTD_SCHEME_CORRECTED ? __fsub_rn(__fadd_rn(a, b), s) : __fsub_rn(2.0f * b, s);
    k.two_dt = 2.0f * dt;
    k.two_tau = 2.0f * tau;
    const float sum = __fadd_rn(dt, tau);
    const float bb = __fsub_rn(sum, dt);
    const float err = __fadd_rn(__fsub_rn(dt, __fsub_rn(sum, bb)), __fsub_rn(tau, bb));
    k.delta = -2.0f * err;
    k.pad0 = k.pad1 = 0.0f;
    return k;
}

// First-order Mur value of one face cell (fdtd_calculations.cu:240-248 and
// mirrors).  rp_self is the slab layer on the face, rp_nbr one cell inwards;
// t_nbr is E^{n+1} at the inner neighbour, s_nbr and s_self are E^n.
__device__ __forceinline__ float mur_value(float dt, float h, float me, float rp_self, float rp_nbr, float t_nbr,
                                           float s_nbr, float s_self)
{
    // every operation rounded on its own, in the reference's order
    // (fdtd_calculations.cu:240-247): no contraction into fused multiply-adds,
    // so each kernel that applies a Mur face gets the same bits
    const float q_self = __fmul_rn(h, sqrtf(__fmul_rn(me, rp_self)));
    const float q_nbr = __fmul_rn(h, sqrtf(__fmul_rn(me, rp_nbr)));
    const float num = __fsub_rn(__fadd_rn(__fmul_rn(__fsub_rn(dt, q_nbr), t_nbr), __fmul_rn(__fadd_rn(dt, q_nbr), s_nbr)),
                                __fmul_rn(__fsub_rn(dt, q_self), s_self));
    return __fmul_rn(__fdiv_rn(1.0f, __fadd_rn(dt, q_self)), num);
}

// mur_value of a face cell whose slab layers hold one value, from that
// value's factors k = (1/(dt+q), dt-q, dt+q, dt-q): the same operations on
// the same operands, so the same bits.
__device__ __forceinline__ float mur_value_k(float4 k, float t_nbr, float s_nbr, float s_self)
{
    return __fmul_rn(k.x, __fsub_rn(__fadd_rn(__fmul_rn(k.y, t_nbr), __fmul_rn(k.z, s_nbr)), __fmul_rn(k.w, s_self)));
}

// The twelve (component, face) sets that updateMurBoundary writes.  For face
// set f, (len_u, len_v) is the extent and (u0, v0) the first coordinate of
// its two in-face axes; `axis` is the face normal (0 x, 1 y, 2 z) and `far`
// selects the face at n-1.
struct MurFace {
    int comp, axis, far;
    int u0, len_u, v0, len_v;  // u is the faster in-face axis (x, else y)
};

__host__ __device__ inline MurFace mur_face(int f, int nx, int ny, int nz)
{
    MurFace m;
    m.comp = f / 4;
    m.far = f & 1;
    const int pair = (f >> 1) & 1;
    if (m.comp == 0) {          // ex: y faces (x 0..nx-2, z 1..nz-2), z faces (x 0..nx-2, y 1..ny-2)
        m.axis = pair ? 2 : 1;
        m.u0 = 0; m.len_u = nx - 1;
        if (m.axis == 1) { m.v0 = 1; m.len_v = nz - 2; }
        else { m.v0 = 1; m.len_v = ny - 2; }
    } else if (m.comp == 1) {   // ey: x faces (y 0..ny-2, z 1..nz-2), z faces (x 1..nx-2, y 0..ny-2)
        m.axis = pair ? 2 : 0;
        if (m.axis == 0) { m.u0 = 0; m.len_u = ny - 1; m.v0 = 1; m.len_v = nz - 2; }
        else { m.u0 = 1; m.len_u = nx - 2; m.v0 = 0; m.len_v = ny - 1; }
    } else {                    // ez: x faces (y 1..ny-2, z 0..nz-2), y faces (x 1..nx-2, z 0..nz-2)
        m.axis = pair ? 1 : 0;
        if (m.axis == 0) { m.u0 = 1; m.len_u = ny - 2; m.v0 = 0; m.len_v = nz - 1; }
        else { m.u0 = 1; m.len_u = nx - 2; m.v0 = 0; m.len_v = nz - 1; }
    }
    return m;
}

struct MurSlabs {
    const float *rpx0, *rpy0, *rpz0, *rpx_end, *rpy_end, *rpz_end;
};

// Applies updateMurBoundary to face set f, in-face position (iu, iv); pitch
// is the row stride of the E arrays (nx when dense).
// eT: E^{n+1} (written), eS: E^n.  fix_ey selects the corrected scheme's
// E^{n+1} term on the ey x = nx-1 face (the reference reads E^n there, :323).
__device__ __forceinline__ void mur_apply(int f, int iu, int iv, int nx, int ny, int nz, int pitch, float dt, float hx,
                                          float hy,
                                          float hz, float me, const MurSlabs &rp, float *t0, float *t1, float *t2,
                                          const float *s0, const float *s1, const float *s2, bool fix_ey)
{
    const MurFace m = mur_face(f, nx, ny, nz);
    if (iu >= m.len_u || iv >= m.len_v)
        return;
    const int u = m.u0 + iu, v = m.v0 + iv;
    int x, y, z, dxn = 0, dyn = 0, dzn = 0;
    float h, rs, rn;
    if (m.axis == 0) {
        x = m.far ? nx - 1 : 0; y = u; z = v; dxn = m.far ? -1 : 1; h = hx;
        const float *slab = m.far ? rp.rpx_end : rp.rpx0;
        const size_t base = ((size_t)z * ny + y) * 2;
        rs = slab[base + (m.far ? 1 : 0)];
        rn = slab[base + (m.far ? 0 : 1)];
    } else if (m.axis == 1) {
        x = u; y = m.far ? ny - 1 : 0; z = v; dyn = m.far ? -1 : 1; h = hy;
        const float *slab = m.far ? rp.rpy_end : rp.rpy0;
        rs = slab[((size_t)z * 2 + (m.far ? 1 : 0)) * nx + x];
        rn = slab[((size_t)z * 2 + (m.far ? 0 : 1)) * nx + x];
    } else {
        x = u; y = v; z = m.far ? nz - 1 : 0; dzn = m.far ? -1 : 1; h = hz;
        const float *slab = m.far ? rp.rpz_end : rp.rpz0;
        rs = slab[((size_t)(m.far ? 1 : 0) * ny + y) * nx + x];
        rn = slab[((size_t)(m.far ? 0 : 1) * ny + y) * nx + x];
    }
    const size_t i = cell_index(x, y, z, pitch, ny);
    const size_t j = cell_index(x + dxn, y + dyn, z + dzn, pitch, ny);
    // component pointers picked with selects (an indexed array would live in local memory)
    const float *S = m.comp == 0 ? s0 : (m.comp == 1 ? s1 : s2);
    float *T = m.comp == 0 ? t0 : (m.comp == 1 ? t1 : t2);
    // fdtd_calculations.cu:323: the ey face at x = nx-1 reads E^n at x-1 in
    // its first term as well.
    const bool quirk = m.comp == 1 && m.axis == 0 && m.far && !fix_ey;
    const float t_nbr = quirk ? S[j] : T[j];
    T[i] = mur_value(dt, h, me, rs, rn, t_nbr, S[j], S[i]);
}

// Indices of one face cell at face coordinates (u, v): the cell, its inward
// neighbour and its two Mur slab entries (self, neighbour).
struct MurCellIdx {
    size_t face, nbr, rs, rn;
};

__device__ __forceinline__ MurCellIdx mur_cell_idx(const MurFace &m, int u, int v, int nx, int ny, int nz, int pitch)
{
    const int ks = m.far ? 1 : 0, kn = m.far ? 0 : 1;
    int x, y, z, dxn = 0, dyn = 0, dzn = 0;
    MurCellIdx c;
    if (m.axis == 0) {
        x = m.far ? nx - 1 : 0; y = u; z = v; dxn = m.far ? -1 : 1;
        c.rs = ((size_t)z * ny + y) * 2 + ks;
        c.rn = ((size_t)z * ny + y) * 2 + kn;
    } else if (m.axis == 1) {
        x = u; y = m.far ? ny - 1 : 0; z = v; dyn = m.far ? -1 : 1;
        c.rs = ((size_t)z * 2 + ks) * nx + x;
        c.rn = ((size_t)z * 2 + kn) * nx + x;
    } else {
        x = u; y = v; z = m.far ? nz - 1 : 0; dzn = m.far ? -1 : 1;
        c.rs = ((size_t)ks * ny + y) * nx + x;
        c.rn = ((size_t)kn * ny + y) * nx + x;
    }
    c.face = cell_index(x, y, z, pitch, ny);
    c.nbr = cell_index(x + dxn, y + dyn, z + dzn, pitch, ny);
    return c;
}

// Operands of one face set: target / source arrays of its component, the
// array its neighbour term reads, its cell size and its slab.
struct MurSet {
    const MurFace m;
    float *T;
    const float *S, *TN, *slab;
    float h;
    __device__ __forceinline__ MurSet(int f, int nx, int ny, int nz, float hx, float hy, float hz, const MurSlabs &rp,
                                      float *t0, float *t1, float *t2, const float *s0, const float *s1,
                                      const float *s2, bool fix_ey)
        : m(mur_face(f, nx, ny, nz))
    {
        S = m.comp == 0 ? s0 : (m.comp == 1 ? s1 : s2);
        T = m.comp == 0 ? t0 : (m.comp == 1 ? t1 : t2);
        const bool quirk = m.comp == 1 && m.axis == 0 && m.far && !fix_ey;  // fdtd_calculations.cu:323
        TN = quirk ? S : T;
        h = m.axis == 0 ? hx : (m.axis == 1 ? hy : hz);
        slab = m.axis == 0 ? (m.far ? rp.rpx_end : rp.rpx0)
               : m.axis == 1 ? (m.far ? rp.rpy_end : rp.rpy0)
                             : (m.far ? rp.rpz_end : rp.rpz0);
    }
};

// mur_apply for K cells of one face set at in-face rows iv0, iv0 + vstride,
// ... below v_end: all loads are issued before any store, so K independent loads per
// array are in flight per thread (face cells are written, their neighbours
// and E^n are only read, so no cell is both).
// UNI: the set's slab holds one value whose factors are kf (no slab loads,
// no square roots or division).
template <int K, bool UNI = false>
__device__ __forceinline__ void mur_apply_k(int f, int iu, int iv0, int vstride, int v_end, int nx, int ny, int nz,
                                            int pitch,
                                            float dt, float hx, float hy, float hz, float me, const MurSlabs &rp,
                                            float *t0, float *t1, float *t2, const float *s0, const float *s1,
                                            const float *s2, bool fix_ey, float4 kf = float4{})
{
    const MurSet ms(f, nx, ny, nz, hx, hy, hz, rp, t0, t1, t2, s0, s1, s2, fix_ey);
    const MurFace &m = ms.m;
    if (iu >= m.len_u)
        return;
    const int u = m.u0 + iu;
    float rs[K], rn[K], tn[K], sn[K], sf[K];
    (void)rs;
    (void)rn;
    size_t face[K];
    bool on[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int iv = iv0 + k * vstride;
        on[k] = iv < m.len_v && iv < v_end;
        const MurCellIdx c = mur_cell_idx(m, u, m.v0 + (on[k] ? iv : 0), nx, ny, nz, pitch);
        face[k] = c.face;
        if (on[k]) {
            if constexpr (!UNI) {
                rs[k] = ms.slab[c.rs];
                rn[k] = ms.slab[c.rn];
            }
            tn[k] = ms.TN[c.nbr];
            sn[k] = ms.S[c.nbr];
            sf[k] = ms.S[c.face];
        }
    }
#pragma unroll
    for (int k = 0; k < K; k++)
        if (on[k]) {
            if constexpr (UNI)
                ms.T[face[k]] = mur_value_k(kf, tn[k], sn[k], sf[k]);
            else
                ms.T[face[k]] = mur_value(dt, ms.h, me, rs[k], rn[k], tn[k], sn[k], sf[k]);
        }
}

// mur_apply for K cells of one face set at flat in-face indices idx0,
// idx0 + stride, ... (row-major over (v, u), below len_u * len_v < 2^31);
// loads before stores as in mur_apply_k.
template <int K, bool UNI = false>
__device__ __forceinline__ void mur_apply_flat_k(int f, unsigned idx0, unsigned stride, int nx, int ny, int nz,
                                                 int pitch, float dt, float hx, float hy, float hz, float me,
                                                 const MurSlabs &rp, float *t0, float *t1, float *t2,
                                                 const float *s0, const float *s1, const float *s2, bool fix_ey,
                                                 unsigned limit = 0, float4 kf = float4{})
{
    const MurSet ms(f, nx, ny, nz, hx, hy, hz, rp, t0, t1, t2, s0, s1, s2, fix_ey);
    const MurFace &m = ms.m;
    if (m.len_u <= 0 || m.len_v <= 0)
        return;
    const unsigned lu = (unsigned)m.len_u;
    unsigned total = lu * (unsigned)m.len_v;
    if (limit > 0 && limit < total)  // only the set's first `limit` cells (rows of u)
        total = limit;
    float rs[K], rn[K], tn[K], sn[K], sf[K];
    size_t face[K];
    bool on[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const unsigned idx = idx0 + (unsigned)k * stride;
        on[k] = idx < total;
        const unsigned i = on[k] ? idx : 0u;
        const MurCellIdx c = mur_cell_idx(m, m.u0 + (int)(i % lu), m.v0 + (int)(i / lu), nx, ny, nz, pitch);
        face[k] = c.face;
        if (on[k]) {
            if constexpr (!UNI) {
                rs[k] = ms.slab[c.rs];
                rn[k] = ms.slab[c.rn];
            }
            tn[k] = ms.TN[c.nbr];
            sn[k] = ms.S[c.nbr];
            sf[k] = ms.S[c.face];
        }
    }
#pragma unroll
    for (int k = 0; k < K; k++)
        if (on[k]) {
            if constexpr (UNI)
                ms.T[face[k]] = mur_value_k(kf, tn[k], sn[k], sf[k]);
            else
                ms.T[face[k]] = mur_value(dt, ms.h, me, rs[k], rn[k], tn[k], sn[k], sf[k]);
        }
}

}  // namespace fdtd
