// strip_unit.cuh -- device side of the compact forms' strip kernels (one
// work unit of the step), shared by the single-solve kernels
// (step_strip.cu) and the persistent batched kernels (batch_strip.cu).
//
// Same update as the compact path of step_fused.cu (H, D increment and
// sources, Debye E and the recursion variable R, the x-face Mur updates),
// with the same arithmetic (cell_math.cuh, so both give the same bits), laid
// out to spend fewer instructions per cell:
//
// * A CTA of W warps owns a 32 x TY column tile (TY = RY * W) and a chunk of
//   z planes; lane l of warp w owns the strip of RY cells x0 + l, rows
//   y0 + w RY .. y0 + w RY + RY - 1.  Along the strip, the E^n rows read for
//   one cell's y + 1 neighbour are the next cell's own, and the D update
//   takes H^{n+1/2} at y - 1 from the previous cell of the strip, so only the
//   strip's first cell reads a row written by another warp.
// * Inputs arrive per plane by TMA tile loads into an S-deep mbarrier ring
//   (E^n with a one-cell halo, H^{n-1/2} with a low x / low y halo, the tile's
//   R, class bytes and, with 16-bit R, the rows' scale words).  Outputs go
//   the same way: each thread writes its results into dense shared-memory
//   tiles, and one thread stores the plane's H^{n+1/2},
//   E^{n+1}, R^{n+1} (and scale words) with TMA stores.  No thread computes a
//   global address per cell.
// * Tiles whose cells, halo included, all lie inside the update ranges of
//   every component, away from the x faces and from sources, take a path
//   without per-cell range tests (CTA-uniform choice, per plane for the
//   first and last planes of the grid); the other tiles take the tested
//   path.
//
// Cells the reference does not update get their old value in the stored tile
// (H^{n+1/2} = H^{n-1/2}; E^{n+1} = E^n, which equals the untouched slot's
// E^{n-1} because such cells are never written; R unchanged, or a zero
// residual with 16-bit R), so whole-tile stores leave them as the z-marching
// kernel leaves them.  The Mur kernel then updates the y and z faces.
#pragma once

#include "cell_math.cuh"
#include "native.cuh"
#include "tma_util.cuh"

namespace fdtd {
namespace strip {

using namespace tma;

constexpr int SX = 32;  // tile width in x: one warp's lanes

template <int RY, int W, bool R16>
struct StripGeo {
    static constexpr int TY = RY * W, NTH = 32 * W;
    static_assert(TY % 4 == 0 && TY <= 32, "tile rows: a multiple of 4 (scale-word boxes) and one lane per row");
    static constexpr int EW = SX + 8, EH = TY + 2;  // E^n box: x0-4 .. x0+35, y0-1 .. y0+TY
    static constexpr int HW = SX + 4, HH = TY + 1;  // H box: x0-4 .. x0+31, y0-1 .. y0+TY-1
    static constexpr int RB = R16 ? 2 : 4;
    static constexpr int E_BYTES = EW * EH * 4, H_BYTES = HW * HH * 4, R_BYTES = SX * TY * RB, M_BYTES = SX * TY;
    static constexpr int X_BYTES = R16 ? TY * 4 : 0;
    // one ring stage
    static constexpr int OFF_E = 0;
    static constexpr int OFF_H = OFF_E + 3 * pad128(E_BYTES);
    static constexpr int OFF_R = OFF_H + 3 * pad128(H_BYTES);
    static constexpr int OFF_X = OFF_R + 3 * pad128(R_BYTES);
    static constexpr int OFF_M = OFF_X + pad128(X_BYTES);
    // x-face tiles: the Mur factors of the tile's rows ([TY] float4) of its
    // face (the near one when the tile holds both)
    static constexpr int F_BYTES = TY * 16;
    static constexpr int OFF_F = pad128(OFF_M + M_BYTES);
    static constexpr int STAGE = pad128(OFF_F + F_BYTES);
    static constexpr unsigned TX_FULL = 3u * E_BYTES + 3u * H_BYTES + 3u * R_BYTES + X_BYTES + M_BYTES;
    static constexpr unsigned TX_PRO = 3u * E_BYTES + 3u * H_BYTES;
    static constexpr unsigned TX_EPI = 3u * E_BYTES;
    // the output tiles (dense 32 x TY): H^{n+1/2}, E^{n+1}, R^{n+1}, scale words
    static constexpr int T_BYTES = SX * TY * 4;
    static constexpr int O_H = 0, O_E = 3 * T_BYTES, O_R = 6 * T_BYTES;
    static constexpr int O_X = O_R + 3 * pad128(R_BYTES);
    // Where the output tiles live: in the plane's own ring stage, over its
    // E^n and H boxes (consumed by the H pass), when they fit below the
    // stage's R tiles; else in an area of their own.  In the stage they cost
    // no shared memory (one more CTA per SM), but the stage's refill waits
    // for its stores to have read them.
    static constexpr bool IN_STAGE = O_X + X_BYTES <= OFF_R;
    static constexpr int OUT = IN_STAGE ? 0 : pad128(O_X + X_BYTES);
    // the thread that issues the TMA stores: thread 0, which also issues the
    // loads, when a stage's refill waits for its stores; else lane 0 of warp 1
    static constexpr int STORE_TID = (W > 1 && !IN_STAGE) ? 32 : 0;
    // H^{n+1/2} hz, hy of every row with the x0-1 column in front ([2][TY][33]),
    // and hz, hx of the row above each warp's first row ([2][W][32]; row
    // y0-1 for warp 0)
    static constexpr int XC = 2 * TY * (SX + 1), XR = 2 * W * SX;
};

// Strip shapes: (cells per thread in y, warps per CTA).  0-2 use 8-row tiles
// (the same shared memory per CTA, 4, 8 or 2 warps), 3 uses 16-row tiles.
constexpr int STRIP_SHAPES = 4;
template <int SHAPE> struct Shape;
// BATCH_CTAS16 / BATCH_CTAS32: resident CTAs per SM the batched kernel is
// built for, with 16-bit and 32-bit R (its register bound; the solve's
// constants come from shared memory there).  Measured on the 64-solve batch:
// shape 0 with 16-bit R runs 2.6 % faster at 5 (no spills) than at 6 (80
// registers, spills), and with 32-bit R shared memory allows 5; shape 1
// spills 136-144 bytes at 5.
template <> struct Shape<0> { static constexpr int RY = 2, W = 4, BATCH_CTAS16 = 5, BATCH_CTAS32 = 5; };
template <> struct Shape<1> { static constexpr int RY = 1, W = 8, BATCH_CTAS16 = 4, BATCH_CTAS32 = 4; };
template <> struct Shape<2> { static constexpr int RY = 4, W = 2, BATCH_CTAS16 = 8, BATCH_CTAS32 = 8; };
template <> struct Shape<3> { static constexpr int RY = 4, W = 4, BATCH_CTAS16 = 2, BATCH_CTAS32 = 2; };

#ifndef FDTD_STRIP_STAGES
#define FDTD_STRIP_STAGES 3
#endif
constexpr int S_SEL = FDTD_STRIP_STAGES;  // ring stages

// Tensor maps of one strip launch over c's buffers for ty-row tiles (false:
// not TMA-addressable).
bool encode_strip_maps(const NativeConsts &c, bool r16, int ty, StripMaps *maps);

template <int RY, int W, int S, bool R16>
constexpr int strip_smem_bytes(int nclasses)
{
    using G = StripGeo<RY, W, R16>;
    return 128 + S * G::STAGE + G::OUT + 4 * (G::XC + G::XR) + ((S * 8 + 15) & ~15) + nclasses * 32;
}

struct StripArgs {
    NativeConsts c;
    int zchunk;
};



__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, uint32_t src, int x, int y, int z)
{
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];"
                 ::"l"(reinterpret_cast<uint64_t>(map)), "r"(src), "r"(x), "r"(y), "r"(z)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One thread arms the stage's barrier and issues the plane's boxes; no_r:
// the tile-plane holds no Debye memory, its R (and scale words) are not
// loaded.  With arm_only (the stall test hook) nothing is issued.  part:
// ISSUE_ALL, or the plane in two parts on one barrier -- ISSUE_HALO arms it
// for the whole plane and issues the E^n and H boxes (the H pass's inputs),
// ISSUE_TILE later issues the classes, R, scale words and x-face Mur
// factors (the E pass's).
enum StripIssuePart { ISSUE_ALL = 0, ISSUE_HALO = 1, ISSUE_TILE = 2 };

// A face tile's Mur factors: rows y0 .. of plane 0 of its x face (the near
// one when a tile of a grid at most 32 cells wide holds both; the far face's
// lanes then read theirs from global memory), nullptr in other tiles; plane z
// lies z * plane float4 further on.  bytes: the rows inside the grid x 16.
struct StripFaces {
    const float4 *src;
    size_t plane;
    uint32_t bytes;
};

template <int RY, int W, bool R16>
__device__ __forceinline__ void strip_issue(const StripMaps &maps, const StripFaces &f, unsigned char *stage,
                                            uint32_t bar, int kind, int x0, int y0, int z, bool arm_only, bool no_r,
                                            int part = ISSUE_ALL)
{
    using G = StripGeo<RY, W, R16>;
    if (part != ISSUE_TILE) {
        const unsigned full = (no_r ? G::TX_FULL - 3u * G::R_BYTES - G::X_BYTES : G::TX_FULL) + (f.src ? f.bytes : 0u);
        mbar_expect_tx(bar, kind == PLANE_FULL ? full : (kind == PLANE_PRO ? G::TX_PRO : G::TX_EPI));
        if (arm_only)
            return;
        for (int c = 0; c < 3; c++)
            tma_load_3d(smem_addr(stage + G::OFF_E + c * pad128(G::E_BYTES)), &maps.m[c], x0 - 4, y0 - 1, z, bar);
        if (kind == PLANE_EPI)
            return;
        for (int c = 0; c < 3; c++)
            tma_load_3d(smem_addr(stage + G::OFF_H + c * pad128(G::H_BYTES)), &maps.m[3 + c], x0 - 4, y0 - 1, z,
                        bar);
        if (part == ISSUE_HALO)
            return;
    }
    if (kind != PLANE_FULL)
        return;
    tma_load_3d(smem_addr(stage + G::OFF_M), &maps.m[9], x0, y0, z, bar);
    if (f.src)
        bulk_load(smem_addr(stage + G::OFF_F), f.src + (size_t)z * f.plane, f.bytes, bar);
    if (no_r)
        return;
    for (int c = 0; c < 3; c++)
        tma_load_3d(smem_addr(stage + G::OFF_R + c * pad128(G::R_BYTES)), &maps.m[6 + c], x0, y0, z, bar);
    if (R16)  // rows y0 .. y0+TY-1 of segment x0 / 32 (y0 * 4 bytes: 16-byte aligned)
        tma_load_3d(smem_addr(stage + G::OFF_X), &maps.m[10], y0, x0 / SX, z, bar);
}

// The constants the strip unit reads.  The single-solve kernel passes its
// NativeConsts parameter (constant bank); the batched kernel keeps this
// smaller copy of the current solve's in shared memory, with the source list
// left in the descriptor.
struct StripConsts {
    int nx, ny, nz;
    float kx, ky, kz, tx, ty, tz;
    int scheme, nsources;
    const int *sources;
    const DebyeCoef *coef;
    int nclasses;
    const float *jz;
    int njz;
    int step;
    int *step_counter;
    int *err;
    int fuse_mur_x;
    const float4 *mur_x;
};

__device__ __forceinline__ void strip_consts(StripConsts &o, const NativeConsts &c)
{
    o.nx = c.nx;
    o.ny = c.ny;
    o.nz = c.nz;
    o.kx = c.kx;
    o.ky = c.ky;
    o.kz = c.kz;
    o.tx = c.tx;
    o.ty = c.ty;
    o.tz = c.tz;
    o.scheme = c.scheme;
    o.nsources = c.nsources;
    o.sources = c.sources;
    o.coef = c.coef;
    o.nclasses = c.nclasses;
    o.jz = c.jz;
    o.njz = c.njz;
    o.step = c.step;
    o.step_counter = c.step_counter;
    o.err = c.err;
    o.fuse_mur_x = c.fuse_mur_x;
    o.mur_x = c.mur_x;
}

// Whether the columns x0..x0+31, rows y0..y0+ty-1, planes zc0..zc1-1 hold a source.
template <class C>
__device__ __forceinline__ bool strip_has_source(const C &c, int x0, int y0, int ty, int zc0, int zc1)
{
    bool any = false;
    for (int s = 0; s < c.nsources; s++) {
        const int sx = c.sources[3 * s], sy = c.sources[3 * s + 1], sz = c.sources[3 * s + 2];
        any |= sx >= x0 && sx < x0 + SX && sy >= y0 && sy < y0 + ty && sz >= zc0 && sz < zc1;
    }
    return any;
}

// A CTA's shared memory: S ring stages, the output tiles, the H exchange
// rows, S barriers, the class table.  The store of a plane's output tiles
// must have read them before the next plane writes them: the storing thread
// waits for that before the next plane's first barrier, so the store has a
// whole H pass to drain.
struct StripSmem {
    unsigned char *stages, *outs;
    float *hnx, *xrw;
    uint64_t *bars;
    DebyeCoef *coef;
};

template <int RY, int W, int S, bool R16>
__device__ __forceinline__ StripSmem strip_smem(unsigned char *smem_raw)
{
    using G = StripGeo<RY, W, R16>;
    StripSmem m;
    m.stages = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    m.outs = m.stages + S * G::STAGE;
    m.hnx = reinterpret_cast<float *>(m.outs + G::OUT);       // [2][TY][33]
    m.xrw = m.hnx + G::XC;                                     // [2][W][32]
    m.bars = reinterpret_cast<uint64_t *>(m.xrw + G::XR);
    m.coef = reinterpret_cast<DebyeCoef *>(reinterpret_cast<unsigned char *>(m.bars) + ((S * 8 + 15) & ~15));
    return m;
}

template <int S>
__device__ __forceinline__ void strip_init_bars(const StripSmem &m)
{
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++)
            mbar_init(smem_addr(&m.bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
}

template <class C>
__device__ __forceinline__ void strip_load_coef(const C &c, DebyeCoef *coef, int nthreads)
{
    const float *src = reinterpret_cast<const float *>(c.coef);
    float *dst = reinterpret_cast<float *>(coef);
    for (int i = threadIdx.x; i < c.nclasses * 8; i += nthreads)
        dst[i] = src[i];
}

// One work unit: column tile (bx, by), z chunk bz of one solve.  The ring's
// stages and barrier phases continue from earlier units of the same CTA (g0
// planes staged before).  memless: bit j set when plane zc0 + j of the tile
// holds no Debye memory.  stall (thread 0 only): leave the second plane's
// copies unissued (test hook).  Returns false when a bounded wait gave up
// (the error flag is raised; the CTA must stop).
template <int RY, int W, int S, bool R16, class C>
__device__ __forceinline__ bool strip_unit(const C &c, const StripMaps &maps, int zchunk, int bx, int by,
                                           int bz, unsigned long long memless, const StripSmem &sm, unsigned g0,
                                           bool stall)
{
    using G = StripGeo<RY, W, R16>;
    constexpr int TY = G::TY;
    float *hnx = sm.hnx, *xrw = sm.xrw;
    const DebyeCoef *coef = sm.coef;
    const int nx = c.nx, ny = c.ny, nz = c.nz;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int x0 = bx * SX, y0 = by * TY;
    const int x = x0 + lane, ry0 = w * RY;  // first row of this thread's strip, relative to y0
    const int zc0 = bz * zchunk, zc1 = min(nz, zc0 + zchunk);
    const int p0 = max(zc0 - 1, 0), plast = min(zc1, nz - 1);
    const int nplanes = plast - p0 + 1;
    const bool unit_src = strip_has_source(c, x0, y0, TY, zc0, zc1);

    auto stage = [&](int k) { return sm.stages + ((g0 + k) % S) * G::STAGE; };
    auto bar = [&](int k) { return smem_addr(&sm.bars[(g0 + k) % S]); };
    auto parity = [&](int k) { return (uint32_t)(((g0 + k) / S) & 1); };
    auto no_r = [&](int z) { return z >= zc0 && ((memless >> (z - zc0)) & 1ull) != 0; };
    // x-face Mur updates (updateMurBoundary ey/ez x faces,
    // fdtd_calculations.cu:280-340) in the tiles that hold x = 0 or nx-1;
    // their per-cell factors arrive with the plane's boxes
    const int mur_bits = mur_x_fused_faces(c);
    const bool face_near = (mur_bits & 1) && x0 == 0;
    const bool face_far_cta = (mur_bits & 2) && x0 <= nx - 1 && nx - 1 < x0 + SX;
    const bool face_cta = face_near || face_far_cta;
    const bool faces_both = face_near && face_far_cta;
    StripFaces faces{nullptr, (size_t)ny, 0u};
    if (face_cta) {
        faces.bytes = (uint32_t)min(TY, ny - y0) * 16u;
        faces.src = face_near ? c.mur_x + y0 : c.mur_x + (size_t)nz * ny + y0;
    }
    if (tid == 0)
        for (int k = 0; k < S && k < nplanes; k++)
            strip_issue<RY, W, R16>(maps, faces, stage(k), bar(k), plane_kind(p0 + k, zc0, zc1), x0, y0, p0 + k,
                                    stall && k == 1, no_r(p0 + k));

    float jz_now = 0.0f;
    if (unit_src) {
        const int n = c.step_counter ? *c.step_counter : c.step;
        const int j = c.scheme == FDTD_SCHEME_CORRECTED ? n : n - n % 3;
        jz_now = (j >= 0 && j < c.njz) ? c.jz[j] : 0.0f;
    }
    const float kx = c.kx, ky = c.ky, kz = c.kz, tcx = c.tx, tcy = c.ty, tcz = c.tz;
    const int cls_max = c.nclasses - 1;
    const bool face_far = x == nx - 1;
    const bool face_lane = x < nx && (((mur_bits & 1) && x == 0) || ((mur_bits & 2) && face_far));
    // every own cell and every halo cell inside the update ranges of all
    // components in x and y, no x face, no source
    const bool xy_inside = x0 >= 1 && x0 + SX - 1 <= nx - 2 && y0 >= 1 && y0 + TY - 1 <= ny - 2 && !face_cta &&
                           !unit_src;

    // Range-tested tiles: each component's update range in x and y per row
    // of the strip (fixed for the unit; the z ranges are per plane).  The
    // tested path computes every update and keeps it where its range holds.
    enum : unsigned { M_HX = 1, M_HY = 2, M_HZ = 4, M_E0 = 8, M_E1 = 16, M_E2 = 32, M_EYZ = 64, M_DOM = 128 };
    unsigned mrow = 0;  // 8 bits per row of the strip
#pragma unroll
    for (int r = 0; r < RY; r++) {
        const int y = y0 + ry0 + r;
        const bool in_dom = x < nx && y < ny;
        const bool xi = x >= 1 && x < nx - 1, yi = y >= 1 && y < ny - 1;
        unsigned m = 0;
        m |= (xi && y < ny - 1) ? M_HX : 0u;
        m |= (x < nx - 1 && yi) ? M_HY : 0u;
        m |= (x < nx - 1 && y < ny - 1) ? M_HZ : 0u;
        m |= (in_dom && x < nx - 1 && yi) ? M_E0 : 0u;
        m |= (in_dom && xi && y < ny - 1) ? M_E1 : 0u;
        m |= (in_dom && xi && yi) ? M_E2 : 0u;
        m |= (in_dom && x >= 1) ? M_EYZ : 0u;
        m |= in_dom ? M_DOM : 0u;
        mrow |= m << (8 * r);
    }
    auto has = [&](int r, unsigned bit) { return ((mrow >> (8 * r)) & bit) != 0u; };

    float hxm[RY], hym[RY];  // H^{n+1/2} x, y of the strip's cells at z-1
#pragma unroll
    for (int r = 0; r < RY; r++)
        hxm[r] = hym[r] = 0.0f;

    auto give_up = [&](int k) {
        if (tid == 0) {
            atomicExch(c.err, 1);
            for (int j = k; j < nplanes && j < k + S; j++)
                mbar_wait(bar(j), parity(j));
        }
        if (tid == G::STORE_TID)
            bulk_wait_all();
        __syncthreads();
    };

    for (int k = 0; k < nplanes; k++) {
        const int z = p0 + k;
        if (z >= zc1)
            break;
        bool ok = true;
        if (k == 0)
            ok = mbar_wait(bar(0), parity(0));
        if (ok && k + 1 < nplanes)
            ok = mbar_wait(bar(k + 1), parity(k + 1));
        const float *EA = reinterpret_cast<const float *>(stage(k) + G::OFF_E);
        const float *EB = reinterpret_cast<const float *>(stage(k + 1) + G::OFF_E);
        const float *HA = reinterpret_cast<const float *>(stage(k) + G::OFF_H);
        constexpr int ES = pad128(G::E_BYTES) / 4, HS = pad128(G::H_BYTES) / 4;
        auto ea = [&](int comp, int r, int cc) { return EA[comp * ES + r * G::EW + cc]; };
        auto eb = [&](int comp, int r, int cc) { return EB[comp * ES + r * G::EW + cc]; };
        auto ha = [&](int comp, int r, int cc) { return HA[comp * HS + r * G::HW + cc]; };
        const bool zlo = z < nz - 1, zmid = z >= 1 && z < nz - 1;
        const bool fast = xy_inside && zmid;  // uniform over the CTA
        const int ec = lane + 4;

        // ---- H^{n+1/2} at plane z on the strip (fdtd_calculations.cu:43-76)
        float ex[RY + 1], ey[RY], ez[RY + 1];
        float hxn[RY], hyn[RY], hzn[RY];
        float ey_nb[RY], ez_nb[RY];  // face lanes: E^n y, z of the x-neighbour (read here: the box is
                                     // refilled before the E pass)
#pragma unroll
        for (int r = 0; r <= RY; r++) {
            ex[r] = ea(0, ry0 + r + 1, ec);
            ez[r] = ea(2, ry0 + r + 1, ec);
        }
#pragma unroll
        for (int r = 0; r < RY; r++) {
            const int er = ry0 + r + 1;
            ey[r] = ea(1, er, ec);
            hxn[r] = ha(0, er, ec);
            hyn[r] = ha(1, er, ec);
            hzn[r] = ha(2, er, ec);
            const int y = y0 + ry0 + r;
            if (face_cta) {
                const int cn = face_far ? ec - 1 : ec + 1;
                ey_nb[r] = ea(1, er, cn);
                ez_nb[r] = ea(2, er, cn);
            }
            if (fast) {
                hxn[r] = cm_h(hxn[r], ky, ez[r + 1], ez[r], ky, eb(1, er, ec), ey[r]);
                hyn[r] = cm_h(hyn[r], kz, eb(0, er, ec), ex[r], kx, ea(2, er, ec + 1), ez[r]);
                hzn[r] = cm_h(hzn[r], kx, ea(1, er, ec + 1), ey[r], ky, ex[r + 1], ex[r]);
            } else {
                const float vx = cm_h(hxn[r], ky, ez[r + 1], ez[r], ky, eb(1, er, ec), ey[r]);
                const float vy = cm_h(hyn[r], kz, eb(0, er, ec), ex[r], kx, ea(2, er, ec + 1), ez[r]);
                const float vz = cm_h(hzn[r], kx, ea(1, er, ec + 1), ey[r], ky, ex[r + 1], ex[r]);
                hxn[r] = has(r, M_HX) && zlo ? vx : hxn[r];
                hyn[r] = has(r, M_HY) && zlo ? vy : hyn[r];
                hzn[r] = has(r, M_HZ) && zmid ? vz : hzn[r];
            }
        }
        if (z < zc0) {  // chunk prologue: only the strip's H x, y at zc0 - 1 are needed
#pragma unroll
            for (int r = 0; r < RY; r++) {
                hxm[r] = hxn[r];
                hym[r] = hyn[r];
            }
            if (__syncthreads_or(!ok)) {
                give_up(k);
                return false;
            }
        } else {
#pragma unroll
            for (int r = 0; r < RY; r++) {
                hnx[(ry0 + r) * (SX + 1) + lane + 1] = hzn[r];
                hnx[(TY + ry0 + r) * (SX + 1) + lane + 1] = hyn[r];
            }
            if (w + 1 < W) {
                xrw[(w + 1) * SX + lane] = hzn[RY - 1];
                xrw[(W + w + 1) * SX + lane] = hxn[RY - 1];
            }
            if (w == 0) {  // row y0 - 1: hx, hz (box row 0)
                const float ex_ = ea(0, 0, ec), ey_ = ea(1, 0, ec), ez_ = ea(2, 0, ec);
                float vx = ha(0, 0, ec), vz = ha(2, 0, ec);
                if (fast) {
                    vx = cm_h(vx, ky, ez[0], ez_, ky, eb(1, 0, ec), ey_);
                    vz = cm_h(vz, kx, ea(1, 0, ec + 1), ey_, ky, ex[0], ex_);
                } else if (y0 >= 1 && x < nx) {
                    if (x >= 1 && x < nx - 1 && zlo)
                        vx = cm_h(vx, ky, ez[0], ez_, ky, eb(1, 0, ec), ey_);
                    if (x < nx - 1 && zmid)
                        vz = cm_h(vz, kx, ea(1, 0, ec + 1), ey_, ky, ex[0], ex_);
                } else {
                    vx = vz = 0.0f;
                }
                xrw[lane] = vz;
                xrw[W * SX + lane] = vx;
            }
            if (w == W - 1 && lane < TY) {  // column x0 - 1: hy, hz of row y0 + lane (box column 3)
                const int er = lane + 1, cc = 3, yy = y0 + lane;
                const float ex_ = ea(0, er, cc), ey_ = ea(1, er, cc), ez_ = ea(2, er, cc);
                float vy = ha(1, er, cc), vz = ha(2, er, cc);
                if (fast) {
                    vy = cm_h(vy, kz, eb(0, er, cc), ex_, kx, ea(2, er, cc + 1), ez_);
                    vz = cm_h(vz, kx, ea(1, er, cc + 1), ey_, ky, ea(0, er + 1, cc), ex_);
                } else if (x0 >= 1 && yy < ny) {
                    if (yy >= 1 && yy < ny - 1 && zlo)
                        vy = cm_h(vy, kz, eb(0, er, cc), ex_, kx, ea(2, er, cc + 1), ez_);
                    if (x0 - 1 < nx - 1 && yy < ny - 1 && zmid)
                        vz = cm_h(vz, kx, ea(1, er, cc + 1), ey_, ky, ea(0, er + 1, cc), ex_);
                } else {
                    vy = vz = 0.0f;
                }
                hnx[lane * (SX + 1)] = vz;
                hnx[(TY + lane) * (SX + 1)] = vy;
            }
            // the CTA decides here whether a wait gave up (nothing has
            // reached global memory from this plane yet)
            // outputs in their own area: the tiles this plane writes were
            // stored one plane ago, and that store has read them by now
            // (checked before the barrier)
            if (!G::IN_STAGE && tid == G::STORE_TID)
                bulk_wait_read<0>();
            if (__syncthreads_or(!ok)) {
                give_up(k);
                return false;
            }
            // outputs in their own area: the H pass has consumed this
            // stage's E^n and H boxes, refill them with plane k + S now, half
            // a plane before the rest
            if (!G::IN_STAGE && tid == 0 && k + S < nplanes) {
                fence_async_shared();
                const int zn = p0 + k + S;
                strip_issue<RY, W, R16>(maps, faces, stage(k + S), bar(k + S), plane_kind(zn, zc0, zc1), x0, y0, zn,
                                        false, no_r(zn), ISSUE_HALO);
            }

            // ---- D increment, sources, E^{n+1} and R^{n+1} on the strip
            const bool plane_no_r = no_r(z);  // uniform: R is +0 on every cell of the tile-plane
            unsigned char *O = G::IN_STAGE ? stage(k) : sm.outs;
            float *OH = reinterpret_cast<float *>(O + G::O_H);
            float *OE = reinterpret_cast<float *>(O + G::O_E);
            const unsigned char *M = stage(k) + G::OFF_M;
            constexpr int TS = SX * TY;  // elements of one dense tile
#pragma unroll
            for (int r = 0; r < RY; r++) {
                const int row = ry0 + r, t = row * SX + lane, y = y0 + row;
                const float hz_xm = hnx[row * (SX + 1) + lane], hy_xm = hnx[(TY + row) * (SX + 1) + lane];
                const float hz_ym = r ? hzn[r - 1] : xrw[w * SX + lane];
                const float hx_ym = r ? hxn[r - 1] : xrw[(W + w) * SX + lane];
                const DebyeCoef kc = coef[min((int)M[t], cls_max)];
                const float k12 = cm_k12(kc);
                float r0, r1, r2;
                float sc = 0.0f;
                unsigned short q0 = 0, q1 = 0, q2 = 0;
                if (plane_no_r) {
                    r0 = r1 = r2 = 0.0f;
                } else if constexpr (R16) {
                    const unsigned short *RT = reinterpret_cast<const unsigned short *>(stage(k) + G::OFF_R);
                    constexpr int RS = pad128(G::R_BYTES) / 2;
                    q0 = RT[t];
                    q1 = RT[RS + t];
                    q2 = RT[2 * RS + t];
                    sc = cm_r16_scale(reinterpret_cast<const uint32_t *>(stage(k) + G::OFF_X)[row]);
                    r0 = cm_r16_r(q0, sc, kc.a, ex[r]);
                    r1 = cm_r16_r(q1, sc, kc.a, ey[r]);
                    r2 = cm_r16_r(q2, sc, kc.a, ez[r]);
                } else {
                    const float *RT = reinterpret_cast<const float *>(stage(k) + G::OFF_R);
                    constexpr int RS = pad128(G::R_BYTES) / 4;
                    r0 = RT[t];
                    r1 = RT[RS + t];
                    r2 = RT[2 * RS + t];
                }
                float en0, en1, en2, rn0, rn1, rn2;
                if (fast) {
                    const float g0 = cm_dinc(tcy, hzn[r], hz_ym, tcz, hyn[r], hym[r]);
                    const float g1 = cm_dinc(tcz, hxn[r], hxm[r], tcx, hzn[r], hz_xm);
                    const float g2 = cm_dinc(tcx, hyn[r], hy_xm, tcy, hxn[r], hx_ym);
                    en0 = cm_e_next(kc, k12, ex[r], g0, r0);
                    en1 = cm_e_next(kc, k12, ey[r], g1, r1);
                    en2 = cm_e_next(kc, k12, ez[r], g2, r2);
                    rn0 = cm_r_next(kc, ex[r], g0);
                    rn1 = cm_r_next(kc, ey[r], g1);
                    rn2 = cm_r_next(kc, ez[r], g2);
                    if constexpr (R16) {
                        rn0 = cm_r16_rho(kc.a, en0, rn0);
                        rn1 = cm_r16_rho(kc.a, en1, rn1);
                        rn2 = cm_r16_rho(kc.a, en2, rn2);
                    }
                } else {
                    const bool ex_on = has(r, M_E0) && zmid;  // also the range of g0
                    const float g0 = ex_on ? cm_dinc(tcy, hzn[r], hz_ym, tcz, hyn[r], hym[r]) : 0.0f;
                    const float g1 =
                        has(r, M_E1) && zmid ? cm_dinc(tcz, hxn[r], hxm[r], tcx, hzn[r], hz_xm) : 0.0f;
                    bool src = false;
                    if (unit_src)
                        for (int s = 0; s < c.nsources; s++)
                            src |= c.sources[3 * s + 2] == z && c.sources[3 * s] == x && c.sources[3 * s + 1] == y;
                    const float d2 = cm_dinc(tcx, hyn[r], hy_xm, tcy, hxn[r], hx_ym);
                    const float g2 = has(r, M_DOM) && ((has(r, M_E2) && zlo) || src)
                                         ? (src ? __fsub_rn(d2, jz_now) : d2)
                                         : 0.0f;
                    const bool eyz_on = has(r, M_EYZ) && z >= 1;
                    // not updated: E keeps E^n, R keeps R^n (16-bit R: residual 0)
                    const float u0 = cm_e_next(kc, k12, ex[r], g0, r0);
                    const float u1 = cm_e_next(kc, k12, ey[r], g1, r1);
                    const float u2 = cm_e_next(kc, k12, ez[r], g2, r2);
                    float s0 = cm_r_next(kc, ex[r], g0), s1 = cm_r_next(kc, ey[r], g1), s2 = cm_r_next(kc, ez[r], g2);
                    if constexpr (R16) {
                        s0 = cm_r16_rho(kc.a, u0, s0);
                        s1 = cm_r16_rho(kc.a, u1, s1);
                        s2 = cm_r16_rho(kc.a, u2, s2);
                    }
                    en0 = ex_on ? u0 : ex[r];
                    en1 = eyz_on ? u1 : ey[r];
                    en2 = eyz_on ? u2 : ez[r];
                    rn0 = ex_on ? s0 : (R16 ? 0.0f : r0);
                    rn1 = eyz_on ? s1 : (R16 ? 0.0f : r1);
                    rn2 = eyz_on ? s2 : (R16 ? 0.0f : r2);
                    if (face_cta) {  // uniform over the CTA: every lane takes part in the shuffles
                        const unsigned all = 0xffffffffu;
                        const float ey_hi = __shfl_down_sync(all, en1, 1), ez_hi = __shfl_down_sync(all, en2, 1);
                        const float ey_lo = __shfl_up_sync(all, en1, 1), ez_lo = __shfl_up_sync(all, en2, 1);
                        if (face_lane && y < ny && zmid) {
                            const float4 mf =
                                faces_both && face_far
                                    ? c.mur_x[((size_t)nz + z) * ny + y]
                                    : reinterpret_cast<const float4 *>(stage(k) + G::OFF_F)[row];
                            auto mur = [&](float tn, float sn, float sf) {
                                return __fmul_rn(mf.x, __fsub_rn(__fadd_rn(__fmul_rn(mf.y, tn), __fmul_rn(mf.z, sn)),
                                                                 __fmul_rn(mf.w, sf)));
                            };
                            if (y <= ny - 2) {  // ey faces: y 0..ny-2, z 1..nz-2
                                // fdtd_calculations.cu:323: the far ey face reads E^n at x-1 in both terms
                                const float tn = face_far ? (c.scheme == FDTD_SCHEME_CORRECTED ? ey_lo : ey_nb[r])
                                                          : ey_hi;
                                en1 = mur(tn, ey_nb[r], ey[r]);
                            }
                            if (y >= 1 && y <= ny - 2)  // ez faces: y 1..ny-2 (z = 0 in the Mur kernel)
                                en2 = mur(face_far ? ez_lo : ez_hi, ez_nb[r], ez[r]);
                        }
                    }
                }
                OH[t] = hxn[r];
                OH[TS + t] = hyn[r];
                OH[2 * TS + t] = hzn[r];
                OE[t] = en0;
                OE[TS + t] = en1;
                OE[2 * TS + t] = en2;
                if (plane_no_r) {
                    // R stays +0: nothing to store
                } else if constexpr (R16) {
                    // one warp is one row segment: every cell of it is
                    // rewritten with the segment's new scale
                    unsigned short h0, h1, h2;
                    const uint32_t b = cm_r16_encode(rn0, rn1, rn2, h0, h1, h2);
                    unsigned short *OR = reinterpret_cast<unsigned short *>(O + G::O_R);
                    constexpr int RS = pad128(G::R_BYTES) / 2;
                    OR[t] = h0;
                    OR[RS + t] = h1;
                    OR[2 * RS + t] = h2;
                    if (lane == 0)
                        reinterpret_cast<uint32_t *>(O + G::O_X)[row] = y < ny ? b : 0u;
                } else {
                    float *OR = reinterpret_cast<float *>(O + G::O_R);
                    constexpr int RS = pad128(G::R_BYTES) / 4;
                    OR[t] = rn0;
                    OR[RS + t] = rn1;
                    OR[2 * RS + t] = rn2;
                }
                hxm[r] = hxn[r];
                hym[r] = hyn[r];
            }
            fence_async_shared();
            __syncthreads();  // stage k consumed, output tiles written
            if (tid == G::STORE_TID) {
                const uint32_t ob = smem_addr(O);
                for (int comp = 0; comp < 3; comp++) {
                    tma_store_3d(&maps.m[11 + comp], ob + G::O_H + comp * G::T_BYTES, x0, y0, z);
                    tma_store_3d(&maps.m[14 + comp], ob + G::O_E + comp * G::T_BYTES, x0, y0, z);
                    if (!plane_no_r)
                        tma_store_3d(&maps.m[6 + comp], ob + G::O_R + comp * pad128(G::R_BYTES), x0, y0, z);
                }
                if (R16 && !plane_no_r)
                    tma_store_3d(&maps.m[10], ob + G::O_X, y0, x0 / SX, z);
                bulk_commit();
                if (G::IN_STAGE)  // the refill below overwrites the tiles
                    bulk_wait_read<0>();
            }
        }
        // refill the stage of plane k with plane k + S: all of it after a
        // prologue plane or with the outputs in the stage, else its classes,
        // R and scale words (the boxes went after the H pass)
        if (tid == 0 && k + S < nplanes) {
            fence_async_shared();
            const int zn = p0 + k + S;
            strip_issue<RY, W, R16>(maps, faces, stage(k + S), bar(k + S), plane_kind(zn, zc0, zc1), x0, y0, zn, false,
                                    no_r(zn), (z < zc0 || G::IN_STAGE) ? ISSUE_ALL : ISSUE_TILE);
        }
    }
    return true;
}

// Planes a unit stages (its ring advance).
__host__ __device__ inline int strip_unit_planes(int nz, int zchunk, int bz)
{
    const int zc0 = bz * zchunk, zc1 = min(nz, zc0 + zchunk);
    return min(zc1, nz - 1) - max(zc0 - 1, 0) + 1;
}

}  // namespace strip
}  // namespace fdtd
