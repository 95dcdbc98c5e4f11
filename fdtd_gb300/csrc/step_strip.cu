// step_strip.cu -- the compact forms' single-pass step over column strips
// (one solve per launch; the unit's work is in strip_unit.cuh), the strip
// shapes, their launchers and the memoryless-plane masks.
#include <algorithm>
#include <cstdlib>
#include <vector>

#include "per_device.h"
#include "strip_unit.cuh"

namespace fdtd {

int strip_zchunk(int nz);

namespace strip {
namespace {

// One solve: CTA (bx, by, bz) processes one unit.
template <int RY, int W, int S, bool R16>
__global__ void __launch_bounds__(32 * W) strip_step_kernel(const __grid_constant__ StripArgs a,
                                                            const __grid_constant__ StripMaps maps)
{
    using G = StripGeo<RY, W, R16>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const StripSmem sm = strip_smem<RY, W, S, R16>(smem_raw);
    const NativeConsts &c = a.c;
    const int x0 = blockIdx.x * SX, y0 = blockIdx.y * G::TY, bz = blockIdx.z;
    const int zc0 = bz * a.zchunk, zc1 = min(c.nz, zc0 + a.zchunk);
    strip_init_bars<S>(sm);
    strip_load_coef(c, sm.coef, G::NTH);
    if (c.overlap_prev) {
        // Launched while the previous step's Mur kernel may still run (it
        // writes E at the faces and reads E at faces and their neighbours in
        // the buffer this launch writes, and advances the step counter): a
        // CTA whose boxes stay two cells clear of every face and that holds
        // no source starts at once, every other CTA waits for that grid.
        const bool clear = x0 - 4 >= 2 && x0 + SX + 3 <= c.nx - 3 && y0 - 1 >= 2 && y0 + G::TY <= c.ny - 3 &&
                           zc0 - 1 >= 2 && zc1 <= c.nz - 3 && !strip_has_source(c, x0, y0, G::TY, zc0, zc1);
        if (!clear)
            asm volatile("griddepcontrol.wait;" ::: "memory");
    }
    __syncthreads();
    bool stall = false;
    if (c.stall_once && blockIdx.x == 0 && blockIdx.y == 0 && bz == 0 && threadIdx.x == 0)
        stall = atomicExch(c.stall_once, 0) != 0;
    const unsigned long long memless =
        c.memless ? c.memless[((size_t)bz * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] : 0ull;
    strip_unit<RY, W, S, R16>(c, maps, a.zchunk, blockIdx.x, blockIdx.y, bz, memless, sm, 0u, stall);
    if (threadIdx.x == G::STORE_TID)
        bulk_wait_all();
}

// ------------------------------------------------------------------ host side

// z chunks of at most 24 planes, for both storage forms: on the
// 512 x 512 x 400 phantom within 0.5 % of the fastest limit in every sweep
// (12, 16, 20, 22, 23, 25, 27, 29, 32, 48 tried; in the latest, 23 and 29
// ran 0.4 % and 0.2 % faster, 25 0.7 % and 20 1.2 % slower)
#ifndef FDTD_STRIP_ZCHUNK
#define FDTD_STRIP_ZCHUNK 24
#endif
static_assert(FDTD_STRIP_ZCHUNK >= 2 && FDTD_STRIP_ZCHUNK <= 64, "a unit's memoryless-plane mask has 64 bits");

template <int SHAPE, bool R16>
int launch_shape(const NativeConsts &c, cudaStream_t s)
{
    constexpr int RY = Shape<SHAPE>::RY, W = Shape<SHAPE>::W;
    using G = StripGeo<RY, W, R16>;
    auto kernel = strip_step_kernel<RY, W, S_SEL, R16>;
    if (c.nclasses < 1 || c.nclasses > FDTD_MAX_CLASSES)
        return FDTD_ERR_INVALID;
    StripArgs a;
    a.c = c;
    if (a.c.memless_rows != G::TY)
        a.c.memless = nullptr;  // masks made for another tile height
    a.zchunk = strip_zchunk(c.nz);
    StripMaps maps;
    if (!encode_strip_maps(c, R16, G::TY, &maps))
        return FDTD_ERR_INVALID;
    static PerDeviceOnce<> smem_opt_in;  // the opt-in holds for the current device only
    int dev = 0;
    const cudaError_t de = cudaGetDevice(&dev);
    if (de != cudaSuccess)
        return (int)de;
    const int so = smem_opt_in.run(dev, [&] {
        return (int)cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         strip_smem_bytes<RY, W, S_SEL, R16>(FDTD_MAX_CLASSES));
    });
    if (so != 0)
        return so < 0 ? FDTD_ERR_INVALID : so;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((c.nx + SX - 1) / SX, (c.ny + G::TY - 1) / G::TY, (c.nz + a.zchunk - 1) / a.zchunk);
    cfg.blockDim = dim3(G::NTH);
    cfg.dynamicSmemBytes = strip_smem_bytes<RY, W, S_SEL, R16>(c.nclasses);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = c.overlap_prev ? 1 : 0;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, a, maps);
    return e == cudaSuccess ? FDTD_OK : (int)e;
}

template <bool R16>
int launch_any(const NativeConsts &c, int shape, cudaStream_t s)
{
    switch (shape) {
    case 0: return launch_shape<0, R16>(c, s);
    case 1: return launch_shape<1, R16>(c, s);
    case 2: return launch_shape<2, R16>(c, s);
    case 3: return launch_shape<3, R16>(c, s);
    default: return FDTD_ERR_INVALID;
    }
}

// Shape of a single solve's step: FDTD_STRIP_SHAPE (0-3) in the environment,
// else the shape measured fastest for the form.
int single_shape(bool r16)
{
    const char *v = std::getenv("FDTD_STRIP_SHAPE");
    if (v && v[0] >= '0' && v[0] < '0' + STRIP_SHAPES && v[1] == 0)
        return v[0] - '0';
    // measured fastest on the 512 x 512 x 400 phantom for both forms: 2 x 4
    // (32-bit R: 1.021 against 1.025 ms per step for 1 x 8)
    (void)r16;
    return 0;
}

}  // namespace

bool encode_strip_maps(const NativeConsts &c, bool r16, int ty, StripMaps *maps)
{
    memset(maps, 0, sizeof *maps);
    auto fn = encode_fn();
    if (!fn || c.pitch % 16 != 0 || !aligned16(c.mat) || (r16 && (!c.r_exp || !aligned16(c.r_exp))))
        return false;
    for (int k = 0; k < 3; k++)
        if (!aligned16(c.e_cur[k]) || !aligned16(c.h_in[k]) || !aligned16(c.d_cur[k]) || !aligned16(c.h_out[k]) ||
            !aligned16(c.e_prev[k]) || c.d_cur[k] != c.d_prev[k])
            return false;
    bool ok = true;
    for (int k = 0; k < 3 && ok; k++) {
        ok &= encode_map(fn, &maps->m[k], c.e_cur[k], false, c.nx, c.ny, c.nz, c.pitch, SX + 8, ty + 2);
        ok &= encode_map(fn, &maps->m[3 + k], c.h_in[k], false, c.nx, c.ny, c.nz, c.pitch, SX + 4, ty + 1);
        if (r16)
            ok &= encode_map_3d(fn, &maps->m[6 + k], c.d_cur[k], CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, c.nx, c.ny, c.nz,
                                (size_t)c.pitch, (size_t)c.pitch * c.ny, SX, ty);
        else
            ok &= encode_map(fn, &maps->m[6 + k], c.d_cur[k], false, c.nx, c.ny, c.nz, c.pitch, SX, ty);
        ok &= encode_map(fn, &maps->m[11 + k], c.h_out[k], false, c.nx, c.ny, c.nz, c.pitch, SX, ty);
        ok &= encode_map(fn, &maps->m[14 + k], c.e_prev[k], false, c.nx, c.ny, c.nz, c.pitch, SX, ty);
    }
    ok = ok && encode_map(fn, &maps->m[9], c.mat, true, c.nx, c.ny, c.nz, c.pitch, SX, ty);
    if (ok && r16) {
        const int rows = r16_rows(c.ny), segs = r16_segments(c.nx);
        ok = encode_map_3d(fn, &maps->m[10], c.r_exp, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, rows, segs, c.nz,
                           (size_t)rows, (size_t)rows * segs, ty, 1);
    }
    return ok;
}

}  // namespace strip

int strip_shape_rows(int shape)
{
    switch (shape) {
    case 0: return strip::Shape<0>::RY * strip::Shape<0>::W;
    case 1: return strip::Shape<1>::RY * strip::Shape<1>::W;
    case 2: return strip::Shape<2>::RY * strip::Shape<2>::W;
    case 3: return strip::Shape<3>::RY * strip::Shape<3>::W;
    default: return 0;
    }
}

int strip_single_shape(bool r16) { return strip::single_shape(r16); }

int strip_zchunk(int nz)
{
    // FDTD_STRIP_ZCHUNK in the environment (2-64 planes) overrides the
    // build's limit; read wherever the launch and the masks are made
    int limit = FDTD_STRIP_ZCHUNK;
    if (const char *v = std::getenv("FDTD_STRIP_ZCHUNK")) {
        const int n = std::atoi(v);
        if (n >= 2 && n <= 64)
            limit = n;
    }
    return zchunk_limited(nz, limit);
}

std::vector<unsigned char> strip_plane_flags(const uint8_t *mat, int nx, int ny, int nz, int pitch, const float *specs,
                                             int nclasses)
{
    constexpr int R8 = 8;
    const int tx = (nx + strip::SX - 1) / strip::SX, t8 = (ny + R8 - 1) / R8;
    bool memless_class[256] = {};
    for (int k = 0; k < nclasses && k < 256; k++)
        memless_class[k] = specs[4 * k + 3] == 0.0f;
    std::vector<unsigned char> flags((size_t)nz * t8 * tx, 0);
    parallel_for(nz, 0, [&](int z) {
        for (int by = 0; by < t8; by++)
            for (int bx = 0; bx < tx; bx++) {
                bool ok = true;
                for (int y = by * R8; y < std::min(ny, by * R8 + R8) && ok; y++) {
                    const uint8_t *row = mat + ((size_t)z * ny + y) * pitch;
                    for (int x = bx * strip::SX; x < std::min(nx, bx * strip::SX + strip::SX); x++)
                        ok &= memless_class[row[x]];
                }
                flags[((size_t)z * t8 + by) * tx + bx] = ok;
            }
    });
    return flags;
}

double strip_unit_masks(const std::vector<unsigned char> &flags, int nx, int ny, int nz, int ty, int zchunk,
                        unsigned long long *masks)
{
    constexpr int R8 = 8;
    const int tx = (nx + strip::SX - 1) / strip::SX, t8 = (ny + R8 - 1) / R8, tyn = (ny + ty - 1) / ty;
    const int chunks = (nz + zchunk - 1) / zchunk, sub = ty / R8;
    double cells = 0.0;
    for (int bz = 0; bz < chunks; bz++)
        for (int by = 0; by < tyn; by++)
            for (int bx = 0; bx < tx; bx++) {
                unsigned long long m = 0;
                const int zc0 = bz * zchunk, zc1 = std::min(nz, zc0 + zchunk);
                for (int z = zc0; z < zc1; z++) {
                    bool ok = true;
                    for (int j = 0; j < sub && by * sub + j < t8; j++)
                        ok &= flags[((size_t)z * t8 + by * sub + j) * tx + bx] != 0;
                    if (ok) {
                        m |= 1ull << (z - zc0);
                        cells += (double)(std::min(nx, bx * strip::SX + strip::SX) - bx * strip::SX) *
                                 (std::min(ny, by * ty + ty) - by * ty);
                    }
                }
                masks[((size_t)bz * tyn + by) * tx + bx] = m;
            }
    return cells / ((double)nx * ny * nz);
}

bool strip_usable(const NativeConsts &c, bool r16)
{
    StripMaps maps;
    return strip::encode_strip_maps(c, r16, 8, &maps);
}

int launch_strip_compact(const NativeConsts &c, cudaStream_t s)
{
    return strip::launch_any<false>(c, strip::single_shape(false), s);
}

int launch_strip_compact16(const NativeConsts &c, cudaStream_t s)
{
    return strip::launch_any<true>(c, strip::single_shape(true), s);
}

}  // namespace fdtd
