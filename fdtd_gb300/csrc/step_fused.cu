// step_fused.cu -- the single-pass step: H, D, sources and the Debye E update
// of one Yee step in one z-marching kernel (with the x-face Mur updates),
// followed by the Mur kernel for the y and z faces.
//
// Each CTA owns a 32 x TY column tile of (x, y) and a chunk of z planes.  Per
// plane it stages, in shared memory, E^n with a one-cell halo on every side,
// H^{n-1/2} with a one-cell halo at low x and low y, and the tile's D^n,
// D^{n-1}, E^{n-1} (D form) or R (compact form) and material classes.  It
// recomputes H^{n+1/2} on its low halo, so that D^{n+1} = D^n + dt curl
// H^{n+1/2} needs no neighbour tile's output; H is double-buffered (read
// H_old, write H_new), E and D are updated in their "prev" slots, R in place.
// Every array is therefore read once and written once per step: 97 bytes per
// cell in the D form (15 floats + 1 byte read, 9 floats written), 73 in the
// compact form (9 + 1 byte read, 9 written).
//
// Staging: with nx a multiple of 16 and 16-byte aligned buffers, one thread
// issues TMA tile loads (cp.async.bulk.tensor.3d) for a whole plane into an
// S-deep ring completed through mbarriers (every wait bounded; a timeout
// raises the plan's error flag and the CTA stops).  Otherwise the same ring is
// filled with 4-byte cp.async copies (zero-filled outside the grid).
//
// Shape (32 x 8 tiles, 3 stages, one issuing thread) is the fastest of the
// variants measured on the 512 x 512 x 400 phantom: 16-row tiles with 2
// stages, 4 stages, all Mur faces inside this kernel, and TMA boxes issued by
// 16 lanes were each slower on the same GPU.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <cstring>

#include "cell_math.cuh"
#include "native.cuh"
#include "per_device.h"
#include "tma_util.cuh"

namespace fdtd {
namespace {

using namespace tma;
static_assert(FTX == FUSED_TILE_X, "x-face Mur fusion assumes 32-column tiles");


// Shared-memory layout of one stage for NT tile arrays of TB-byte elements
// (9 floats: D^n, D^{n-1}, E^{n-1} of the D form; 3 floats: R of the compact
// form; 3 FP16 residuals of the compact form with 16-bit R, which also
// stages its TY scale words, XB bytes).
template <int TY, int NT = 9, int TB = 4, int XB = 0>
struct Geo {
    static constexpr int EW = FTX + 8, EH = TY + 2;   // E^n box: x0-4 .. x0+TX+3, y0-1 .. y0+TY
    static constexpr int HW = FTX + 4, HH = TY + 1;   // H box: x0-4 .. x0+TX-1, y0-1 .. y0+TY-1
    static constexpr int E_BYTES = EW * EH * 4, H_BYTES = HW * HH * 4, T_BYTES = FTX * TY * TB, M_BYTES = FTX * TY;
    static constexpr int OFF_E = 0;
    static constexpr int OFF_H = OFF_E + 3 * pad128(E_BYTES);
    static constexpr int OFF_T = OFF_H + 3 * pad128(H_BYTES);
    static constexpr int OFF_X = OFF_T + NT * pad128(T_BYTES);
    static constexpr int OFF_M = OFF_X + pad128(XB);
    static constexpr int STAGE = pad128(OFF_M + M_BYTES);
    static constexpr int HNW = FTX + 1, HNH = TY + 1;  // H^{n+1/2} plane incl. low halo
    static constexpr int HN_BYTES = pad128(3 * HNW * HNH * 4);
    // expected transaction bytes per plane kind
    static constexpr unsigned TX_FULL = 3u * E_BYTES + 3u * H_BYTES + unsigned(NT) * T_BYTES + XB + M_BYTES;
    static constexpr unsigned TX_PRO = 3u * E_BYTES + 3u * H_BYTES;
    static constexpr unsigned TX_EPI = 3u * E_BYTES;
};

// Stage geometry of a form.
template <int TY, bool COMPACT, bool R16>
using GeoOf = Geo<TY, COMPACT ? 3 : 9, R16 ? 2 : 4, R16 ? TY * 4 : 0>;

struct FusedArgs {
    NativeConsts c;
    int zchunk;
};

// TMA: one thread arms the stage's barrier and issues the plane's boxes.
// With arm_only (the stall test hook) the barrier expects the plane's bytes
// but no copy is issued.  The tile maps follow the six halo maps, then the
// classes, then (16-bit R) the scale words.
template <int TY, int NT = 9, int TB = 4, int XB = 0>
__device__ void issue_plane_tma(const FusedMaps &maps, unsigned char *stage, uint32_t bar, int kind, int x0, int y0,
                                int z, bool arm_only = false)
{
    using G = Geo<TY, NT, TB, XB>;
    const unsigned bytes = kind == PLANE_FULL ? G::TX_FULL : (kind == PLANE_PRO ? G::TX_PRO : G::TX_EPI);
    mbar_expect_tx(bar, bytes);
    if (arm_only)
        return;
    for (int c = 0; c < 3; c++)
        tma_load_3d(smem_addr(stage + G::OFF_E + c * pad128(G::E_BYTES)), &maps.m[c], x0 - 4, y0 - 1, z, bar);
    if (kind == PLANE_EPI)
        return;
    for (int c = 0; c < 3; c++)
        tma_load_3d(smem_addr(stage + G::OFF_H + c * pad128(G::H_BYTES)), &maps.m[3 + c], x0 - 4, y0 - 1, z, bar);
    if (kind == PLANE_PRO)
        return;
    for (int k = 0; k < NT; k++)
        tma_load_3d(smem_addr(stage + G::OFF_T + k * pad128(G::T_BYTES)), &maps.m[6 + k], x0, y0, z, bar);
    tma_load_3d(smem_addr(stage + G::OFF_M), &maps.m[6 + NT], x0, y0, z, bar);
    if (XB > 0)  // scale words of rows y0 .. y0+TY-1 of segment x0 / 32 (y0 * 4 bytes: 16-byte aligned)
        tma_load_3d(smem_addr(stage + G::OFF_X), &maps.m[7 + NT], y0, x0 / FTX, z, bar);
}

// Generic: every thread copies part of each box with 4-byte cp.async
// (zero-filled outside the grid); the material classes are read separately,
// and so are 16-bit R and its scale words (no tiles staged for them).
template <int TY, int NT = 9, int TB = 4, int XB = 0>
__device__ void issue_plane_generic(const NativeConsts &c, unsigned char *stage, int kind, int x0, int y0, int z,
                                    int tid)
{
    using G = Geo<TY, NT, TB, XB>;
    constexpr int NTH = FTX * TY;
    const int nx = c.nx, ny = c.ny, pitch = c.pitch;
    const size_t plane = (size_t)pitch * ny;
    auto box = [&](const float *base, uint32_t dst, int xs, int ys, int w, int h) {
        for (int i = tid; i < w * h; i += NTH) {
            const int gx = xs + i % w, gy = ys + i / w;
            const bool ok = gx >= 0 && gx < nx && gy >= 0 && gy < ny;
            const float *src = ok ? base + (size_t)z * plane + (size_t)gy * pitch + gx : base;
            cp_async4(dst + 4u * i, src, ok);
        }
    };
    for (int k = 0; k < 3; k++)
        box(c.e_cur[k], smem_addr(stage + G::OFF_E + k * pad128(G::E_BYTES)), x0 - 4, y0 - 1, G::EW, G::EH);
    if (kind == PLANE_EPI)
        return;
    for (int k = 0; k < 3; k++)
        box(c.h_in[k], smem_addr(stage + G::OFF_H + k * pad128(G::H_BYTES)), x0 - 4, y0 - 1, G::HW, G::HH);
    if (kind == PLANE_PRO)
        return;
    const float *tiles[9] = {c.d_cur[0], c.d_cur[1], c.d_cur[2], c.d_prev[0], c.d_prev[1],
                             c.d_prev[2], c.e_prev[0], c.e_prev[1], c.e_prev[2]};
    if (TB == 4)
        for (int k = 0; k < NT; k++)
            box(tiles[k], smem_addr(stage + G::OFF_T + k * pad128(G::T_BYTES)), x0, y0, FTX, TY);
}

// ---------------------------------------------------------------- the kernel

// Whether the unit's columns x0..x0+31, rows y0..y0+ty-1 and planes
// zc0..zc1-1 hold a source cell.
__device__ __forceinline__ bool unit_has_source(const NativeConsts &c, int x0, int y0, int ty, int zc0, int zc1)
{
    bool any = false;
    for (int s = 0; s < c.nsources; s++) {
        const int sx = c.sources[3 * s], sy = c.sources[3 * s + 1], sz = c.sources[3 * s + 2];
        any |= sx >= x0 && sx < x0 + FTX && sy >= y0 && sy < y0 + ty && sz >= zc0 && sz < zc1;
    }
    return any;
}

// ---- 16-bit R (layout: r16_segments / r16_rows / r16_words)

// Index of the scale word of row y, segment bx, plane z.
__device__ __forceinline__ size_t r16_word(const NativeConsts &c, int z, int bx, int y)
{
    return ((size_t)z * r16_segments(c.nx) + bx) * r16_rows(c.ny) + y;
}

// One work unit: the column tile (bx, by) and z chunk bz of one solve.  The
// stage ring and its barriers continue from earlier units of the same CTA:
// g0 counts the planes this CTA has staged before.  Returns false when a
// bounded wait gave up (the error flag is set; the CTA must stop).  stall
// (read by thread 0 only): leave the second plane's copies unissued.
template <int TY, int S, bool TMA, bool COMPACT = false, bool R16 = false>
__device__ __forceinline__ bool fused_unit(const NativeConsts &c, const FusedMaps &maps, int zchunk, int bx, int by,
                                           int bz, unsigned char *smem, const DebyeCoef *coef, uint64_t *bars,
                                           unsigned g0, bool stall = false)
{
    static_assert(COMPACT || !R16, "16-bit R is a compact-form layout");
    constexpr int NT = COMPACT ? 3 : 9, TB = R16 ? 2 : 4, XB = R16 ? TY * 4 : 0;
    using G = Geo<TY, NT, TB, XB>;
    const int nx = c.nx, ny = c.ny, nz = c.nz;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * FTX + tx;
    const int x0 = bx * FTX, y0 = by * TY;
    const int x = x0 + tx, y = y0 + ty;
    const int zc0 = bz * zchunk, zc1 = min(nz, zc0 + zchunk);
    const int p0 = max(zc0 - 1, 0), plast = min(zc1, nz - 1);
    const int nplanes = plast - p0 + 1;

    float *hn = reinterpret_cast<float *>(smem + S * G::STAGE);
    auto stage = [&](int k) { return smem + ((g0 + k) % S) * G::STAGE; };
    auto bar = [&](int k) { return smem_addr(&bars[(g0 + k) % S]); };
    auto parity = [&](int k) { return ((g0 + k) / S) & 1u; };

    // prologue: fill the ring
    for (int k = 0; k < S; k++) {
        if (k < nplanes) {
            const int z = p0 + k;
            if (TMA) {
                if (tid == 0)
                    issue_plane_tma<TY, NT, TB, XB>(maps, stage(k), bar(k), plane_kind(z, zc0, zc1), x0, y0, z,
                                            stall && k == 1);
            } else {
                issue_plane_generic<TY, NT, TB, XB>(c, stage(k), plane_kind(z, zc0, zc1), x0, y0, z, tid);
            }
        }
        if (!TMA)
            cp_async_commit();
    }

    // source of this step (sample index n - n%3 in the reference scheme),
    // read only by units that hold a source cell
    float jz_now = 0.0f;
    const bool unit_src = unit_has_source(c, x0, y0, TY, zc0, zc1);
    // planes p0 + d (d < 66: chunks hold at most 64 planes) at which this
    // thread's column holds a source: bit d of src_lo, or bit d - 64 of src_hi
    unsigned long long src_lo = 0ull;
    unsigned src_hi = 0u;
    if (unit_src) {
        for (int s = 0; s < c.nsources; s++) {
            const int d = c.sources[3 * s + 2] - p0;
            if (c.sources[3 * s] == x && c.sources[3 * s + 1] == y && d >= 0 && d < 96) {
                if (d < 64)
                    src_lo |= 1ull << d;
                else
                    src_hi |= 1u << (d - 64);
            }
        }
        const int n = c.step_counter ? *c.step_counter : c.step;
        const int j = c.scheme == FDTD_SCHEME_CORRECTED ? n : n - n % 3;
        jz_now = (j >= 0 && j < c.njz) ? c.jz[j] : 0.0f;
    }

    const bool in_dom = x < nx && y < ny;
    const size_t plane = (size_t)c.pitch * ny;  // elements between z planes
    const size_t col = (size_t)y * c.pitch + x;
    const float kx = c.kx, ky = c.ky, kz = c.kz, tcx = c.tx, tcy = c.ty, tcz = c.tz;
    const int cls_max = c.nclasses - 1;  // the table holds nclasses entries; larger codes read the last
    // x-face Mur updates (updateMurBoundary ey/ez x faces, fdtd_calculations.cu:280-340)
    // for the tiles that hold x = 0 or x = nx-1: the face lane takes E^{n+1}
    // of its x-neighbour from the adjacent lane by a shuffle, E^n from the
    // staged box and the cell's four Mur factors from a register prefetch.
    const int mur_bits = mur_x_fused_faces(c);
    const bool face_cta = ((mur_bits & 1) && x0 == 0) || ((mur_bits & 2) && x0 <= nx - 1 && nx - 1 < x0 + FTX);
    const bool face_far = x == nx - 1;
    const bool face_lane = x < nx && y < ny && (((mur_bits & 1) && x == 0) || ((mur_bits & 2) && face_far));
    const float4 *mur_col = face_lane ? c.mur_x + (size_t)(face_far ? 1 : 0) * nz * ny + y : nullptr;
    float4 mf = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // factors of the face cell at the current plane
    auto load_mf = [&](int zz) {
        if (face_lane && zz >= 1 && zz <= nz - 2)
            mf = mur_col[(size_t)zz * ny];
    };
    load_mf(zc0);
    float hxm = 0.0f, hym = 0.0f;  // H^{n+1/2} of this column at z-1
    uint8_t mat_next = 0;
    if (!TMA && in_dom && zc0 < nz)
        mat_next = c.mat[(size_t)zc0 * plane + col];

    // a bounded wait gave up: raise the error flag, let the copies in flight
    // land (bounded) and leave; called by every thread after one CTA-wide
    // decision, so no thread is left at a barrier
    auto give_up = [&](int k) {
        if (tid == 0) {
            atomicExch(c.err, 1);
            for (int j = k; j < nplanes && j < k + S; j++)
                mbar_wait(bar(j), parity(j));
        }
        __syncthreads();
    };
    for (int k = 0; k < nplanes; k++) {
        const int z = p0 + k;
        if (z >= zc1)
            break;
        // planes k and k+1 resident
        bool ok = true;
        if (TMA) {
            if (k == 0)
                ok = mbar_wait(bar(0), parity(0));
            if (ok && k + 1 < nplanes)
                ok = mbar_wait(bar(k + 1), parity(k + 1));
            // the CTA decides at its next barrier (below): until then it only
            // reads shared memory
        } else {
            cp_async_wait<S - 2>();
            __syncthreads();
        }
        const float *EA = reinterpret_cast<const float *>(stage(k) + G::OFF_E);
        const float *EB = reinterpret_cast<const float *>(stage(k + 1) + G::OFF_E);
        const float *HA = reinterpret_cast<const float *>(stage(k) + G::OFF_H);
        constexpr int ES = pad128(G::E_BYTES) / 4, HS = pad128(G::H_BYTES) / 4, TS = pad128(G::T_BYTES) / 4;
        auto ea = [&](int comp, int r, int cc) { return EA[comp * ES + r * G::EW + cc]; };
        auto eb = [&](int comp, int r, int cc) { return EB[comp * ES + r * G::EW + cc]; };
        auto ha = [&](int comp, int r, int cc) { return HA[comp * HS + r * G::HW + cc]; };
        auto hnr = [&](int comp, int r, int cc) -> float & { return hn[(comp * G::HNH + r) * G::HNW + cc]; };

        const bool zlo = z < nz - 1, zmid = z >= 1 && z < nz - 1;
        // ---- H^{n+1/2} at plane z, own cell (fdtd_calculations.cu:43-76)
        float hxn = 0.0f, hyn = 0.0f, hzn = 0.0f;
        if (in_dom) {
            const int r = ty + 1, cc = tx + 4;
            const float ex_ = ea(0, r, cc), ey_ = ea(1, r, cc), ez_ = ea(2, r, cc);
            hxn = ha(0, r, cc);
            hyn = ha(1, r, cc);
            hzn = ha(2, r, cc);
            if (x >= 1 && x < nx - 1 && y < ny - 1 && zlo)
                hxn = cm_h(hxn, ky, ea(2, r + 1, cc), ez_, ky, eb(1, r, cc), ey_);
            if (x < nx - 1 && y >= 1 && y < ny - 1 && zlo)
                hyn = cm_h(hyn, kz, eb(0, r, cc), ex_, kx, ea(2, r, cc + 1), ez_);
            if (x < nx - 1 && y < ny - 1 && zmid)
                hzn = cm_h(hzn, kx, ea(1, r, cc + 1), ey_, ky, ea(0, r + 1, cc), ex_);
        }
        if (z < zc0) {  // chunk prologue: only this column's H at zc0 - 1 is needed
            hxm = hxn;
            hym = hyn;
        } else {
            if (in_dom) {
                hnr(0, ty + 1, tx + 1) = hxn;
                hnr(1, ty + 1, tx + 1) = hyn;
                hnr(2, ty + 1, tx + 1) = hzn;
            }
            // low-x halo column: hy, hz at x0 - 1 for the TY rows, one lane of the
            // last warp per row (the low-y row below is warp 0's)
            if (ty == TY - 1 && tx < TY) {
                const int row = tx, yy = y0 + row;
                if (x0 >= 1 && yy < ny) {
                    const int r = row + 1, cc = 3;  // x0 - 1
                    const float ex_ = ea(0, r, cc), ey_ = ea(1, r, cc), ez_ = ea(2, r, cc);
                    const int xh = x0 - 1;
                    float v = ha(1, r, cc);
                    if (yy >= 1 && yy < ny - 1 && zlo)
                        v = cm_h(v, kz, eb(0, r, cc), ex_, kx, ea(2, r, cc + 1), ez_);
                    hnr(1, row + 1, 0) = v;
                    v = ha(2, r, cc);
                    if (xh < nx - 1 && yy < ny - 1 && zmid)
                        v = cm_h(v, kx, ea(1, r, cc + 1), ey_, ky, ea(0, r + 1, cc), ex_);
                    hnr(2, row + 1, 0) = v;
                }
            }
            // low-y halo row: hx, hz at y - 1 (decision point below: nothing
            // is written to global memory before it)
            if (ty == 0 && y >= 1 && x < nx) {
                const int r = 0, cc = tx + 4;  // y - 1
                const float ex_ = ea(0, r, cc), ey_ = ea(1, r, cc), ez_ = ea(2, r, cc);
                float v = ha(0, r, cc);
                if (x >= 1 && x < nx - 1 && zlo)
                    v = cm_h(v, ky, ea(2, r + 1, cc), ez_, ky, eb(1, r, cc), ey_);
                hnr(0, 0, tx + 1) = v;
                v = ha(2, r, cc);
                if (x < nx - 1 && zmid)
                    v = cm_h(v, kx, ea(1, r, cc + 1), ey_, ky, ea(0, r + 1, cc), ex_);
                hnr(2, 0, tx + 1) = v;
            }
            if (TMA) {
                if (__syncthreads_or(!ok)) {
                    give_up(k);
                    return false;
                }
            } else {
                __syncthreads();
            }

            float ey_new = 0.0f, ez_new = 0.0f;  // this lane's E^{n+1} y, z (for the x-face lanes)
            if constexpr (COMPACT) {
            const size_t i = (size_t)z * plane + col;
            float rho0 = 0.0f, rho1 = 0.0f, rho2 = 0.0f;  // 16-bit R: the residuals to store (0 where not updated)
            if (in_dom) {
                const int t = ty * FTX + tx;
                float r0, r1, r2;    // R^n (32-bit R)
                unsigned short q0, q1, q2;  // stored residuals (FP16 bits) and their segment's word (16-bit R)
                uint32_t w;
                if constexpr (R16) {
                    if (TMA) {
                        const unsigned short *T = reinterpret_cast<const unsigned short *>(stage(k) + G::OFF_T);
                        constexpr int TS16 = pad128(G::T_BYTES) / 2;
                        q0 = T[t];
                        q1 = T[TS16 + t];
                        q2 = T[2 * TS16 + t];
                        w = reinterpret_cast<const uint32_t *>(stage(k) + G::OFF_X)[ty];
                    } else {
                        q0 = reinterpret_cast<const unsigned short *>(c.d_cur[0])[i];
                        q1 = reinterpret_cast<const unsigned short *>(c.d_cur[1])[i];
                        q2 = reinterpret_cast<const unsigned short *>(c.d_cur[2])[i];
                        w = c.r_exp[r16_word(c, z, bx, y)];
                    }
                } else {
                    const float *T = reinterpret_cast<const float *>(stage(k) + G::OFF_T);
                    r0 = T[0 * TS + t];
                    r1 = T[1 * TS + t];
                    r2 = T[2 * TS + t];
                }
                uint8_t cls;
                if (TMA) {
                    cls = (stage(k) + G::OFF_M)[t];
                } else {
                    cls = mat_next;
                    if (z + 1 < zc1)
                        mat_next = c.mat[i + plane];
                }
                if (x >= 1 && x < nx - 1 && y < ny - 1 && zlo)
                    c.h_out[0][i] = hxn;
                if (x < nx - 1 && y >= 1 && y < ny - 1 && zlo)
                    c.h_out[1][i] = hyn;
                if (x < nx - 1 && y < ny - 1 && zmid)
                    c.h_out[2][i] = hzn;

                // ---- this step's D increment dD = dt curl H^{n+1/2} (and the sources)
                const bool xi = x >= 1 && x < nx - 1, yi = y >= 1 && y < ny - 1;
                const bool dx_on = x < nx - 1 && yi && zmid;
                const bool dy_on = xi && y < ny - 1 && zmid;
                const bool dz_on = xi && yi && zlo;
                float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f;
                if (dx_on)
                    g0 = cm_dinc(tcy, hzn, hnr(2, ty, tx + 1), tcz, hyn, hym);
                if (dy_on)
                    g1 = cm_dinc(tcz, hxn, hxm, tcx, hzn, hnr(2, ty + 1, tx));
                // the per-cell test over the source list, in units that hold a
                // source only, measured faster than the column mask in this form
                // (which needs three more registers of the 48)
                bool src = false;
                if (unit_src)
                    for (int s = 0; s < c.nsources; s++)
                        src |= c.sources[3 * s + 2] == z && c.sources[3 * s] == x && c.sources[3 * s + 1] == y;
                if (dz_on || src) {
                    g2 = cm_dinc(tcx, hyn, hnr(1, ty + 1, tx), tcy, hxn, hnr(0, ty, tx + 1));
                    if (src)
                        g2 = __fsub_rn(g2, jz_now);
                }

                // ---- E^{n+1} = c (d E^n + (2 dt + 2 tau) dD + R^n),  R^{n+1} = -a E^n - 2 tau dD
                const bool ex_on = x < nx - 1 && yi && zmid;
                const bool eyz_on = x >= 1 && z >= 1;
                if (ex_on || eyz_on) {
                    const DebyeCoef kc = coef[min((int)cls, cls_max)];
                    const float k12 = cm_k12(kc);
                    const int r = ty + 1, cc = tx + 4;
                    if constexpr (R16) {  // R^n = rho - a E^n
                        const float sc = cm_r16_scale(w);
                        r0 = cm_r16_r(q0, sc, kc.a, ea(0, r, cc));
                        r1 = cm_r16_r(q1, sc, kc.a, ea(1, r, cc));
                        r2 = cm_r16_r(q2, sc, kc.a, ea(2, r, cc));
                    }
                    if (ex_on) {
                        const float e = ea(0, r, cc);
                        const float en = cm_e_next(kc, k12, e, g0, r0);
                        const float rn = cm_r_next(kc, e, g0);
                        c.e_prev[0][i] = en;
                        if constexpr (R16) {
                            rho0 = cm_r16_rho(kc.a, en, rn);
                        } else {
                            c.d_prev[0][i] = rn;
                        }
                    }
                    if (eyz_on) {
                        const float e1 = ea(1, r, cc), e2 = ea(2, r, cc);
                        ey_new = cm_e_next(kc, k12, e1, g1, r1);
                        ez_new = cm_e_next(kc, k12, e2, g2, r2);
                        c.e_prev[1][i] = ey_new;
                        const float rn1 = cm_r_next(kc, e1, g1);
                        c.e_prev[2][i] = ez_new;
                        const float rn2 = cm_r_next(kc, e2, g2);
                        if constexpr (R16) {
                            rho1 = cm_r16_rho(kc.a, ey_new, rn1);
                            rho2 = cm_r16_rho(kc.a, ez_new, rn2);
                        } else {
                            c.d_prev[1][i] = rn1;
                            c.d_prev[2][i] = rn2;
                        }
                    }
                }
            }
            if constexpr (R16) {
                // every cell of the row segment is rewritten with the
                // segment's new scale (cells whose E is never updated
                // store 0)
                if (y < ny) {  // uniform over the warp: one warp is one row
                    unsigned short h0, h1, h2;
                    const uint32_t b = cm_r16_encode(rho0, rho1, rho2, h0, h1, h2);
                    if (x < nx) {
                        reinterpret_cast<unsigned short *>(c.d_prev[0])[i] = h0;
                        reinterpret_cast<unsigned short *>(c.d_prev[1])[i] = h1;
                        reinterpret_cast<unsigned short *>(c.d_prev[2])[i] = h2;
                    }
                    if (tx == 0)
                        c.r_exp[r16_word(c, z, bx, y)] = b;
                }
            }
            } else {
            if (in_dom) {
                const size_t i = (size_t)z * plane + col;
                const float *T = reinterpret_cast<const float *>(stage(k) + G::OFF_T);
                const int t = ty * FTX + tx;
                const float dn0 = T[0 * TS + t], dn1 = T[1 * TS + t], dn2 = T[2 * TS + t];
                const float dp0 = T[3 * TS + t], dp1 = T[4 * TS + t], dp2 = T[5 * TS + t];
                const float ep0 = T[6 * TS + t], ep1 = T[7 * TS + t], ep2 = T[8 * TS + t];
                uint8_t cls;
                if (TMA) {
                    cls = (stage(k) + G::OFF_M)[t];
                } else {
                    cls = mat_next;
                    if (z + 1 < zc1)
                        mat_next = c.mat[i + plane];
                }
                // H^{n+1/2}: write the updated components
                if (x >= 1 && x < nx - 1 && y < ny - 1 && zlo)
                    c.h_out[0][i] = hxn;
                if (x < nx - 1 && y >= 1 && y < ny - 1 && zlo)
                    c.h_out[1][i] = hyn;
                if (x < nx - 1 && y < ny - 1 && zmid)
                    c.h_out[2][i] = hzn;

                // ---- D^{n+1} (fdtd_calculations.cu:96-121) and sources (:198-211)
                const bool xi = x >= 1 && x < nx - 1, yi = y >= 1 && y < ny - 1;
                const bool dx_on = x < nx - 1 && yi && zmid;
                const bool dy_on = xi && y < ny - 1 && zmid;
                bool dz_on = xi && yi && zlo;
                float d0 = dp0, d1 = dp1, d2 = dp2;
                if (dx_on)
                    d0 = dn0 + tcy * (hzn - hnr(2, ty, tx + 1)) - tcz * (hyn - hym);
                if (dy_on)
                    d1 = dn1 + tcz * (hxn - hxm) - tcx * (hzn - hnr(2, ty + 1, tx));
                const int dz = z - p0;
                const bool src = dz < 64 ? ((src_lo >> dz) & 1ull) : ((src_hi >> (dz - 64)) & 1u);
                if (dz_on || src) {
                    d2 = dn2 + tcx * (hyn - hnr(1, ty + 1, tx)) - tcy * (hxn - hnr(0, ty, tx + 1));
                    if (src)
                        d2 = d2 - jz_now;
                    dz_on = true;
                }
                if (dx_on) c.d_prev[0][i] = d0;
                if (dy_on) c.d_prev[1][i] = d1;
                if (dz_on) c.d_prev[2][i] = d2;

                // ---- Debye E^{n+1} (fdtd_calculations.cu:146-183)
                const bool ex_on = x < nx - 1 && yi && zmid;
                const bool eyz_on = x >= 1 && z >= 1;
                if (ex_on || eyz_on) {
                    const DebyeCoef kc = coef[min((int)cls, cls_max)];
                    const int r = ty + 1, cc = tx + 4;
                    if (ex_on)
                        c.e_prev[0][i] = debye_update(kc, ea(0, r, cc), ep0, d0, dn0, dp0);
                    if (eyz_on) {
                        ey_new = debye_update(kc, ea(1, r, cc), ep1, d1, dn1, dp1);
                        ez_new = debye_update(kc, ea(2, r, cc), ep2, d2, dn2, dp2);
                        c.e_prev[1][i] = ey_new;
                        c.e_prev[2][i] = ez_new;
                    }
                }
            }
            }
            if (face_cta) {  // uniform over the CTA: every lane takes part in the shuffles
                const unsigned all = 0xffffffffu;
                const float ey_hi = __shfl_down_sync(all, ey_new, 1), ez_hi = __shfl_down_sync(all, ez_new, 1);
                const float ey_lo = __shfl_up_sync(all, ey_new, 1), ez_lo = __shfl_up_sync(all, ez_new, 1);
                if (face_lane && zmid) {
                    const size_t i = (size_t)z * plane + col;
                    const int r = ty + 1, cc = tx + 4, cn = face_far ? cc - 1 : cc + 1;
                    // mur_value with the factors precomputed, same roundings
                    auto mur = [&](float tn, float sn, float sf) {
                        return __fmul_rn(mf.x, __fsub_rn(__fadd_rn(__fmul_rn(mf.y, tn), __fmul_rn(mf.z, sn)),
                                                         __fmul_rn(mf.w, sf)));
                    };
                    if (y <= ny - 2) {  // ey faces: y 0..ny-2, z 1..nz-2
                        // fdtd_calculations.cu:323: the far ey face reads E^n at x-1 in both terms
                        const float tn = face_far ? (c.scheme == FDTD_SCHEME_CORRECTED ? ey_lo : ea(1, r, cn)) : ey_hi;
                        c.e_prev[1][i] = mur(tn, ea(1, r, cn), ea(1, r, cc));
                    }
                    if (y >= 1 && y <= ny - 2)  // ez faces: y 1..ny-2, z 0..nz-2 (z = 0 in the Mur kernel)
                        c.e_prev[2][i] = mur(face_far ? ez_lo : ez_hi, ea(2, r, cn), ea(2, r, cc));
                }
                load_mf(z + 1);
            }
            hxm = hxn;
            hym = hyn;
        }
        if (TMA && z < zc0) {  // the chunk prologue plane has no other decision point
            if (__syncthreads_or(!ok)) {
                give_up(k);
                return false;
            }
        } else {
            __syncthreads();  // stage k and hn fully consumed
        }
        // refill the stage of plane k with plane k + S
        const int kn = k + S;
        if (TMA) {
            if (tid == 0 && kn < nplanes) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const int zn = p0 + kn;
                issue_plane_tma<TY, NT, TB, XB>(maps, stage(kn), bar(kn), plane_kind(zn, zc0, zc1), x0, y0, zn);
            }
        } else {
            if (kn < nplanes) {
                const int zn = p0 + kn;
                issue_plane_generic<TY, NT, TB, XB>(c, stage(kn), plane_kind(zn, zc0, zc1), x0, y0, zn, tid);
            }
            cp_async_commit();
        }
    }
    if (!TMA)
        cp_async_wait<0>();
    return true;
}

// Shared-memory layout of a CTA: S stages, the H^{n+1/2} plane, S barriers,
// then the class table (the launch sizes it for the solve's classes, so a
// small table leaves room for more resident CTAs).
template <int S>
__host__ __device__ constexpr int bars_bytes() { return (S * 8 + 15) & ~15; }

template <int S, class G>
__host__ __device__ constexpr int fused_smem_bytes(int nclasses)
{
    return 128 + S * G::STAGE + G::HN_BYTES + bars_bytes<S>() + nclasses * (int)sizeof(DebyeCoef);
}

template <int S, bool TMA, class G>
__device__ __forceinline__ void fused_cta_setup(unsigned char *smem, DebyeCoef **coef, uint64_t **bars)
{
    *bars = reinterpret_cast<uint64_t *>(smem + S * G::STAGE + G::HN_BYTES);
    *coef = reinterpret_cast<DebyeCoef *>(smem + S * G::STAGE + G::HN_BYTES + bars_bytes<S>());
    const int tid = threadIdx.y * FTX + threadIdx.x;
    if (TMA && tid == 0) {
        for (int s = 0; s < S; s++)
            mbar_init(smem_addr(&(*bars)[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
}

__device__ __forceinline__ void load_coef(const NativeConsts &c, DebyeCoef *coef, int nthreads)
{
    const float *src = reinterpret_cast<const float *>(c.coef);
    float *dst = reinterpret_cast<float *>(coef);
    const int tid = threadIdx.y * FTX + threadIdx.x;
    for (int i = tid; i < c.nclasses * 8; i += nthreads)
        dst[i] = src[i];
}

// One solve: CTA (bx, by, bz) processes one unit.
template <int TY, int S, bool TMA, bool COMPACT, bool R16 = false>
__global__ void __launch_bounds__(FTX *TY) fused_step_kernel(const __grid_constant__ FusedArgs a,
                                                             const __grid_constant__ FusedMaps maps)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    DebyeCoef *coef;
    uint64_t *bars;
    fused_cta_setup<S, TMA, GeoOf<TY, COMPACT, R16>>(smem, &coef, &bars);
    load_coef(a.c, coef, FTX * TY);
    const int bz = blockIdx.z;
    if (a.c.overlap_prev) {
        // Launched while the previous step's Mur kernel may still run.  That
        // kernel writes the E face cells and reads E at faces and their
        // neighbours (indices 0, 1, n-2, n-1 of each axis) in the buffer this
        // launch overwrites, and it advances the step counter.  A CTA whose
        // boxes (x0-4 .. x0+35, y0-1 .. y0+TY, planes zc0-1 .. zc1) stay two
        // cells clear of every face and that holds no source cell touches
        // none of that; every other CTA waits for the Mur grid to finish.
        const int x0 = blockIdx.x * FTX, y0 = blockIdx.y * TY;
        const int zc0 = bz * a.zchunk, zc1 = min(a.c.nz, zc0 + a.zchunk);
        const bool clear = x0 - 4 >= 2 && x0 + FTX + 3 <= a.c.nx - 3 && y0 - 1 >= 2 && y0 + TY <= a.c.ny - 3 &&
                           zc0 - 1 >= 2 && zc1 <= a.c.nz - 3 && !unit_has_source(a.c, x0, y0, TY, zc0, zc1);
        if (!clear)
            asm volatile("griddepcontrol.wait;" ::: "memory");
    }
    __syncthreads();
    bool stall = false;
    if (TMA && a.c.stall_once && blockIdx.x == 0 && blockIdx.y == 0 && bz == 0 && threadIdx.x == 0 &&
        threadIdx.y == 0)
        stall = atomicExch(a.c.stall_once, 0) != 0;
    fused_unit<TY, S, TMA, COMPACT, R16>(a.c, maps, a.zchunk, blockIdx.x, blockIdx.y, bz, smem, coef, bars, 0u,
                                         stall);
}

// Many solves: persistent CTAs take work units from a counter; a unit's solve
// descriptor supplies the constants (copied to shared memory) and tensor maps
// (read by TMA from device memory).  Units of finished solves are skipped.
// The compact forms are bounded for 4 resident CTAs per SM (the 64-solve
// workload ran 4.8 % faster than with 5: fewer units in flight, more
// registers per thread; with 16-bit R 11 % faster than with 3 or 5).
template <int TY, int S, bool COMPACT, bool R16 = false>
__global__ void __launch_bounds__(FTX *TY, COMPACT ? 4 : 3) batch_step_kernel(const BatchDesc *__restrict__ descs, int nsolves,
                                                             int total_units, int *work_counter)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    __shared__ NativeConsts s_c;
    __shared__ int s_unit, s_solve;
    DebyeCoef *coef;
    uint64_t *bars;
    fused_cta_setup<S, true, GeoOf<TY, COMPACT, R16>>(smem, &coef, &bars);
    const int tid = threadIdx.y * FTX + threadIdx.x;
    int loaded = -1;
    unsigned g = 0;
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
                for (int i = tid; i < (int)(sizeof(NativeConsts) / 4); i += FTX * TY)
                    dst[i] = src[i];
            }
            if (sv != loaded)
                load_coef(d.c[par], coef, FTX * TY);
            __syncthreads();
            loaded = sv;
            const int local = u - d.unit_begin;
            const int per_z = d.tiles_x * d.tiles_y;
            const int bz = local / per_z, rem = local % per_z;
            const int by = rem / d.tiles_x, bx = rem % d.tiles_x;
            const int zc0 = bz * d.zchunk, zc1 = min(s_c.nz, zc0 + d.zchunk);
            const int nplanes = min(zc1, s_c.nz - 1) - max(zc0 - 1, 0) + 1;
            if (!fused_unit<TY, S, true, COMPACT, R16>(s_c, d.maps[par], d.zchunk, bx, by, bz, smem, coef, bars, g))
                return;
            g += (unsigned)nplanes;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) batch_mur_kernel(const BatchDesc *__restrict__ descs,
                                                        const BatchMurBlock *__restrict__ blocks)
{
    const BatchMurBlock b = blocks[blockIdx.x];
    const BatchDesc &d = descs[b.solve];
    const int n = *d.c[0].step_counter;
    if (n >= d.steps_target)
        return;
    const NativeConsts &c = d.c[n & 1];
    // BATCH_MUR_CELLS cells from b.first: thread t takes first + t + k * 256
    // (faces of batched solves hold < 2^31 cells)
    const MurFace m = mur_face(b.face, c.nx, c.ny, c.nz);
    const int slab = m.axis + 3 * m.far;
    if ((c.mur_uniform >> slab) & 1) {  // one value in the set's slab: its factors
        const float4 kf = make_float4(c.mur_k[slab][0], c.mur_k[slab][1], c.mur_k[slab][2], c.mur_k[slab][3]);
        mur_apply_flat_k<BATCH_MUR_CELLS / 256, true>(b.face, (unsigned)b.first + threadIdx.x, 256u, c.nx, c.ny, c.nz,
                                                      c.pitch, c.dt, c.hx, c.hy, c.hz, c.me, c.rp, c.e_prev[0],
                                                      c.e_prev[1], c.e_prev[2], c.e_cur[0], c.e_cur[1], c.e_cur[2],
                                                      c.scheme == FDTD_SCHEME_CORRECTED, (unsigned)b.limit, kf);
        return;
    }
    mur_apply_flat_k<BATCH_MUR_CELLS / 256>(b.face, (unsigned)b.first + threadIdx.x, 256u, c.nx, c.ny, c.nz, c.pitch,
                                            c.dt, c.hx, c.hy, c.hz, c.me, c.rp, c.e_prev[0], c.e_prev[1],
                                            c.e_prev[2], c.e_cur[0], c.e_cur[1], c.e_cur[2],
                                            c.scheme == FDTD_SCHEME_CORRECTED, (unsigned)b.limit);
}

__global__ void batch_advance_kernel(const BatchDesc *__restrict__ descs, int nsolves, int *work_counter)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0)
        *work_counter = 0;
    if (s < nsolves) {
        int *ctr = descs[s].c[0].step_counter;
        if (*ctr < descs[s].steps_target)
            *ctr += 1;
    }
}

// ------------------------------------------------------------------ host side

// Tile rows and ring depth (build-time constants; 8 x 3 measured fastest).
#ifndef FDTD_TILE_ROWS
#define FDTD_TILE_ROWS 8
#endif
#ifndef FDTD_RING_STAGES
#define FDTD_RING_STAGES 3
#endif
// Largest z chunk of the compact form.  Its CTAs run at about 1.3x the D
// form's cell rate; with chunks of 24 planes or more its DRAM throughput fell
// on grids above 100 M cells (0.86 of the copy bandwidth at 24 planes, 0.80
// at 64) while 16-20 planes held 0.96-0.99 from 105 M to 537 M cells.
#ifndef FDTD_COMPACT_ZCHUNK
#define FDTD_COMPACT_ZCHUNK 16
#endif
constexpr int TY_SEL = FDTD_TILE_ROWS;
constexpr int S_SEL = FDTD_RING_STAGES;


template <bool TMA, bool COMPACT, bool R16 = false>
int launch_fused_impl(const FusedArgs &a, const FusedMaps &maps, cudaStream_t s)
{
    auto kernel = fused_step_kernel<TY_SEL, S_SEL, TMA, COMPACT, R16>;
    using G = GeoOf<TY_SEL, COMPACT, R16>;
    if (a.c.nclasses < 1 || a.c.nclasses > FDTD_MAX_CLASSES)
        return FDTD_ERR_INVALID;
    // the shared-memory opt-in holds for the current device only
    static PerDeviceOnce<> smem_opt_in;
    int dev = 0;
    cudaError_t de = cudaGetDevice(&dev);
    if (de != cudaSuccess)
        return (int)de;
    const int so = smem_opt_in.run(dev, [&] {
        return (int)cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         fused_smem_bytes<S_SEL, G>(FDTD_MAX_CLASSES));
    });
    if (so != 0)
        return so < 0 ? FDTD_ERR_INVALID : so;
    const int smem = fused_smem_bytes<S_SEL, G>(a.c.nclasses);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((a.c.nx + FTX - 1) / FTX, (a.c.ny + TY_SEL - 1) / TY_SEL, (a.c.nz + a.zchunk - 1) / a.zchunk);
    cfg.blockDim = dim3(FTX, TY_SEL);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = a.c.overlap_prev ? 1 : 0;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, a, maps);
    return e == cudaSuccess ? FDTD_OK : (int)e;
}

}  // namespace

// nz split into equal chunks of at most max_planes planes
int zchunk_limited(int nz, int max_planes)
{
    const int chunks = (nz + max_planes - 1) / max_planes;
    return (nz + chunks - 1) / chunks;
}

#ifndef FDTD_ZCHUNK
#define FDTD_ZCHUNK 64
#endif
static_assert(FDTD_ZCHUNK >= 4 && FDTD_ZCHUNK <= 64, "a unit's per-thread source mask covers 66 planes");

int fused_zchunk(int nz)
{
    // about 64 planes per CTA: enough CTAs per wave on 152 SMs, little
    // prologue/epilogue traffic at chunk borders.  At most 64: a unit's
    // per-thread source mask covers 66 planes.
    return zchunk_limited(nz, FDTD_ZCHUNK);
}

int compact_zchunk(int nz) { return zchunk_limited(nz, FDTD_COMPACT_ZCHUNK); }

bool fused_uses_tma(const NativeConsts &c)
{
    if (c.pitch % 16 != 0 || !encode_fn())
        return false;
    for (int k = 0; k < 3; k++)
        if (!aligned16(c.e_cur[k]) || !aligned16(c.h_in[k]) || !aligned16(c.d_cur[k]) || !aligned16(c.d_prev[k]) ||
            !aligned16(c.e_prev[k]))
            return false;
    return aligned16(c.mat);
}

// Tensor maps of one step: E^n and H^{n-1/2} halo boxes (0-5), the tile
// arrays (D form: D^n, D^{n-1}, E^{n-1} at 6-14; compact form: R at 6-8) and
// the class volume after them; with 16-bit R (FP16 tiles at 6-8) the
// scale words at 10 (box: one segment's TY rows).
bool encode_step_maps(const NativeConsts &c, bool compact, FusedMaps *maps, bool r16)
{
    memset(maps, 0, sizeof *maps);
    if (!fused_uses_tma(c) || (r16 && (!compact || !c.r_exp || !aligned16(c.r_exp))))
        return false;
    auto fn = encode_fn();
    using G = Geo<TY_SEL>;
    const float *const *tiles[3] = {c.d_cur, c.d_prev, c.e_prev};
    const int ntile_sets = compact ? 1 : 3;
    bool ok = true;
    for (int k = 0; k < 3 && ok; k++) {
        ok &= encode_map(fn, &maps->m[k], c.e_cur[k], false, c.nx, c.ny, c.nz, c.pitch, G::EW, G::EH);
        ok &= encode_map(fn, &maps->m[3 + k], c.h_in[k], false, c.nx, c.ny, c.nz, c.pitch, G::HW, G::HH);
        for (int t = 0; t < ntile_sets; t++) {
            if (r16)  // pitch % 16 == 0: rows of 2-byte values keep 16-byte strides
                ok &= encode_map_3d(fn, &maps->m[6 + k], tiles[t][k], CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, c.nx, c.ny,
                                    c.nz, (size_t)c.pitch, (size_t)c.pitch * c.ny, FTX, TY_SEL);
            else
                ok &= encode_map(fn, &maps->m[6 + 3 * t + k], tiles[t][k], false, c.nx, c.ny, c.nz, c.pitch, FTX,
                                 TY_SEL);
        }
    }
    ok = ok && encode_map(fn, &maps->m[6 + 3 * ntile_sets], c.mat, true, c.nx, c.ny, c.nz, c.pitch, FTX, TY_SEL);
    if (ok && r16) {
        const int rows = r16_rows(c.ny), segs = r16_segments(c.nx);
        ok = encode_map_3d(fn, &maps->m[10], c.r_exp, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, rows, segs, c.nz,
                           (size_t)rows, (size_t)rows * segs, TY_SEL, 1);
    }
    return ok;
}

bool encode_fused_maps(const NativeConsts &c, FusedMaps *maps) { return encode_step_maps(c, false, maps); }

int fused_tile_height() { return TY_SEL; }

// Shared memory of the persistent batch kernel: tiles of the form and a class
// table for the batch's largest class count.
template <bool COMPACT, bool R16 = false>
int batch_smem(int nclasses) { return fused_smem_bytes<S_SEL, GeoOf<TY_SEL, COMPACT, R16>>(nclasses); }

// The batch kernel's shared-memory opt-in on the current device (it holds
// for that device only): made on the first use there.
template <bool COMPACT, bool R16 = false>
int batch_opt_in()
{
    auto kernel = batch_step_kernel<TY_SEL, S_SEL, COMPACT, R16>;
    static PerDeviceOnce<> smem_opt_in;
    int dev = 0;
    const cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return (int)e;
    const int so = smem_opt_in.run(dev, [&] {
        return (int)cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         batch_smem<COMPACT, R16>(FDTD_MAX_CLASSES));
    });
    return so < 0 ? FDTD_ERR_INVALID : so;
}

template <bool COMPACT, bool R16 = false>
int batch_ctas_impl(int nclasses)
{
    auto kernel = batch_step_kernel<TY_SEL, S_SEL, COMPACT, R16>;
    batch_opt_in<COMPACT, R16>();
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, FTX * TY_SEL, batch_smem<COMPACT, R16>(nclasses));
    return sms * (per_sm > 0 ? per_sm : 1);
}

int batch_persistent_ctas(bool compact, int nclasses, bool r16)
{
    if (r16)
        return batch_ctas_impl<true, true>(nclasses);
    return compact ? batch_ctas_impl<true>(nclasses) : batch_ctas_impl<false>(nclasses);
}

int launch_batch_step(const BatchLaunch &b, cudaStream_t s)
{
    if (b.max_classes < 1 || b.max_classes > FDTD_MAX_CLASSES)
        return FDTD_ERR_INVALID;
    cudaError_t e = cudaSuccess;
    if (b.strip) {
        const int st = launch_batch_strip(b, s);
        if (st != FDTD_OK)
            return st;
    } else {
    const int oi = b.r16 ? batch_opt_in<true, true>() : (b.compact ? batch_opt_in<true>() : batch_opt_in<false>());
    if (oi != FDTD_OK)
        return oi;
    if (b.r16)
        batch_step_kernel<TY_SEL, S_SEL, true, true>
            <<<b.persistent_ctas, dim3(FTX, TY_SEL), batch_smem<true, true>(b.max_classes), s>>>(
                b.descs, b.nsolves, b.total_units, b.work_counter);
    else if (b.compact)
        batch_step_kernel<TY_SEL, S_SEL, true>
            <<<b.persistent_ctas, dim3(FTX, TY_SEL), batch_smem<true>(b.max_classes), s>>>(
                b.descs, b.nsolves, b.total_units, b.work_counter);
    else
        batch_step_kernel<TY_SEL, S_SEL, false>
            <<<b.persistent_ctas, dim3(FTX, TY_SEL), batch_smem<false>(b.max_classes), s>>>(
                b.descs, b.nsolves, b.total_units, b.work_counter);
    e = cudaGetLastError();
    }
    if (e == cudaSuccess && b.nmur_blocks > 0) {
        batch_mur_kernel<<<b.nmur_blocks, 256, 0, s>>>(b.descs, b.mur_blocks);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        batch_advance_kernel<<<(b.nsolves + 255) / 256, 256, 0, s>>>(b.descs, b.nsolves, b.work_counter);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? FDTD_OK : (int)e;
}

int launch_h_de_fused(const NativeConsts &c, cudaStream_t s)
{
    FusedArgs a;
    a.c = c;
    a.zchunk = fused_zchunk(c.nz);
    FusedMaps maps;
    if (encode_step_maps(c, false, &maps))
        return launch_fused_impl<true, false>(a, maps, s);
    return launch_fused_impl<false, false>(a, maps, s);
}

// The compact forms run the strip kernel (step_strip.cu) wherever its TMA
// loads and stores can address the arrays, else the z-marching kernel here;
// FDTD_COMPACT_STEP=zmarch in the environment selects the z-marching kernel
// everywhere (both give the same bits; used to cross-check them).
static bool strip_selected(const NativeConsts &c, bool r16)
{
    const char *v = std::getenv("FDTD_COMPACT_STEP");
    return !(v && std::strcmp(v, "zmarch") == 0) && strip_usable(c, r16);
}

int launch_h_e_compact(const NativeConsts &c, cudaStream_t s)
{
    if (c.d_cur[0] != c.d_prev[0] || c.d_cur[1] != c.d_prev[1] || c.d_cur[2] != c.d_prev[2])
        return FDTD_ERR_INVALID;  // R is updated in place
    if (strip_selected(c, false))
        return launch_strip_compact(c, s);
    static_assert(FDTD_COMPACT_ZCHUNK >= 4, "z chunks hold at least four planes");
    FusedArgs a;
    a.c = c;
    a.zchunk = compact_zchunk(c.nz);  // the compact form reads no source-plane mask
    FusedMaps maps;
    if (encode_step_maps(c, true, &maps))
        return launch_fused_impl<true, true>(a, maps, s);
    return launch_fused_impl<false, true>(a, maps, s);
}

int launch_h_e_compact16(const NativeConsts &c, cudaStream_t s)
{
    if (c.d_cur[0] != c.d_prev[0] || c.d_cur[1] != c.d_prev[1] || c.d_cur[2] != c.d_prev[2] || !c.r_exp)
        return FDTD_ERR_INVALID;  // R and its scale words are updated in place
    if (strip_selected(c, true))
        return launch_strip_compact16(c, s);
    FusedArgs a;
    a.c = c;
    a.zchunk = compact_zchunk(c.nz);
    FusedMaps maps;
    if (encode_step_maps(c, true, &maps, true))
        return launch_fused_impl<true, true, true>(a, maps, s);
    return launch_fused_impl<false, true, true>(a, maps, s);
}

int launch_step(const NativeConsts &c0, cudaStream_t s)
{
    NativeConsts c = c0;
    c.fuse_mur_x = 1;
    int st = launch_h_de_fused(c, s);
    if (st == FDTD_OK)
        st = launch_mur(c, s);
    return st;
}

int launch_step_compact(const NativeConsts &c0, cudaStream_t s)
{
    NativeConsts c = c0;
    c.fuse_mur_x = 1;
    int st = launch_h_e_compact(c, s);
    if (st == FDTD_OK)
        st = launch_mur(c, s);
    return st;
}

int launch_step_compact16(const NativeConsts &c0, cudaStream_t s)
{
    NativeConsts c = c0;
    c.fuse_mur_x = 1;
    int st = launch_h_e_compact16(c, s);
    if (st == FDTD_OK)
        st = launch_mur(c, s);
    return st;
}

int step_kernels(int kernel_kind, const NativeConsts &, StepKernel *out, int max)
{
    static const StepKernel single[] = {{"fused_step", launch_h_de_fused}, {"mur", launch_mur}};
    static const StepKernel compact[] = {{"compact_step", launch_h_e_compact}, {"mur", launch_mur}};
    static const StepKernel compact16[] = {{"compact16_step", launch_h_e_compact16}, {"mur", launch_mur}};
    static const StepKernel two[] = {{"h", launch_h}, {"de", launch_de}, {"mur", launch_mur}};
    const StepKernel *src = kernel_kind == FDTD_KERNEL_SINGLE_PASS ? single
                            : kernel_kind == FDTD_KERNEL_COMPACT   ? compact
                            : kernel_kind == FDTD_KERNEL_COMPACT_R16 ? compact16
                                                                     : two;
    const int n = kernel_kind == FDTD_KERNEL_TWO_PASS ? 3 : 2;
    for (int k = 0; k < n && k < max; k++)
        out[k] = src[k];
    return n;
}

}  // namespace fdtd
