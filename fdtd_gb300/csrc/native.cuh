// native.cuh -- plan object and kernel argument block of the native path.
#pragma once

#include <cuda.h>

#include <vector>

#include "device_common.cuh"

struct fdtd_plan {
    int device = 0;
    int nx = 0, ny = 0, nz = 0;
    float dt = 0, dx = 0, dy = 0, dz = 0, mu0 = 0, eps0 = 0;
    int scheme = FDTD_SCHEME_REFERENCE;
    int nclasses = 0;
    int nsources = 0;
    int sources[3 * FDTD_MAX_SOURCES] = {};
    int njz = 0;
    std::vector<fdtd::DebyeCoef> host_coef;
    char *d_block = nullptr;              // one allocation for everything below
    fdtd::DebyeCoef *d_coef = nullptr;    // nclasses entries
    float *d_jz = nullptr;                // FDTD_JZ_LEN entries
    fdtd::MurSlabs rp{};                  // six Mur slabs
    float4 *d_mur_x = nullptr;            // x-face Mur coefficients, [face][z][y] (see mur_x_coef)
    float mur_k[6][4] = {};               // per Mur slab holding one value: the factors of every cell
    int mur_uniform = 0;                  // bit s: slab s (NativeConsts::mur_k order) holds one value
    int *d_err = nullptr;                 // device error flag
    int *d_stall = nullptr;               // test hook word (NativeConsts::stall_once)
    bool pooled = false;                  // d_block comes from a stream-ordered pool (plan_create_on)
};

namespace fdtd {

// Kernel argument block (passed by value).
struct NativeConsts {
    int nx, ny, nz;
    int pitch;             // elements between consecutive rows (nx for dense arrays)
    float kx, ky, kz;      // dt / (mu0 d{x,y,z}) of the H update
    float tx, ty, tz;      // dt / d{x,y,z} of the D update
    float dt, hx, hy, hz;  // time step and cell sizes (Mur)
    float me;              // mu0 * eps0 (Mur)
    int scheme;
    int nsources;
    int sources[3 * FDTD_MAX_SOURCES];
    const DebyeCoef *coef;
    int nclasses;
    const float *jz;
    int njz;
    MurSlabs rp;
    int step;              // step index n when step_counter is null
    int *step_counter;     // device step index (graph replay), may be null
    int *err;              // device error flag (a bounded wait gave up)
    int *stall_once;       // test hook, may be null: when set, the first CTA of the next single-pass
                           // launch clears it and arms one plane's barrier without issuing its
                           // copies, so that CTA's bounded wait runs out (raises *err)
    int overlap_prev;      // single-pass launch may start while the previous step's Mur kernel runs
                           // (programmatic dependent launch; only where that kernel precedes it)
    int fuse_mur_x;        // the single-pass kernel applies the x-face Mur updates and the Mur
                           // kernel of the same step skips them (set for both launches or neither)
    const float4 *mur_x;   // per x-face cell: 1/(dt+q_self), dt-q_nbr, dt+q_nbr, dt-q_self, [face][z][y]
    uint32_t *r_exp;       // compact form with 16-bit R: the segment scale words (see r16_words),
                           // and d_cur == d_prev hold the FP16 residuals; null in the other forms
    const float *h_in[3];
    float *h_out[3];
    const float *e_cur[3];
    float *e_prev[3];
    const float *d_cur[3];
    float *d_prev[3];
    const uint8_t *mat;
    // compact forms, strip kernel: per unit (tile x, tile y, z chunk) a bit
    // per plane of the chunk whose tile holds only classes without
    // relaxation (R stays +0 there: not loaded, not stored); may be null
    const unsigned long long *memless;
    int memless_rows;      // tile rows the masks were made for (other tile heights ignore them)
    // Mur slabs that hold one value (slab s: x0, y0, z0, x_end, y_end, z_end,
    // i.e. face normal s % 3, far face s / 3; set when every entry of both
    // layers of the slab is that value, as for slabs made from the default
    // material): bit s of mur_uniform, and the factors 1/(dt+q), dt-q, dt+q,
    // dt-q of its every face cell, q = h sqrt(me rp), each rounded as
    // mur_value rounds it
    float mur_k[6][4];
    int mur_uniform;
};

NativeConsts make_consts(const fdtd_plan *p, const fdtd_native_fields *f, int n);

// Checks every class index of a dense volume against nclasses (host threads
// over z planes); returns, where the pointers are not null, a hash of the
// volume and its largest class index.
int scan_material(const uint8_t *mat, int nx, int ny, int nz, int nclasses, unsigned long long *hash,
                  int *top_class = nullptr);

// x-face Mur updates done by the single-pass kernel: bit 0 the x = 0 face,
// bit 1 the x = nx-1 face (only when x = nx-2 lies in the same 32-column
// tile, so one warp holds both cells).  The Mur kernel skips these, except
// for the ez row at z = 0, whose x = 1 neighbour the single-pass kernel does
// not update.
constexpr int FUSED_TILE_X = 32;
template <class C>
__host__ __device__ inline int mur_x_fused_faces(const C &c)
{
    return c.fuse_mur_x && c.mur_x ? (1 | ((c.nx - 1) % FUSED_TILE_X != 0 ? 2 : 0)) : 0;
}

int launch_h(const NativeConsts &c, cudaStream_t s);
int launch_de(const NativeConsts &c, cudaStream_t s);
int launch_mur(const NativeConsts &c, cudaStream_t s);
// Single-pass step: H, D, sources and E in one z-marching kernel, then Mur.
int launch_step(const NativeConsts &c, cudaStream_t s);

// Compact form with R stored in 16 bits.  What is stored is the residual
// rho_k = R_k^{n+1} + a E_k^{n+1} (a = 2 eps0 eps_inf tau of the cell's
// class), which the next step turns back into R_k = rho_k - a E_k with the
// FP32 E it reads anyway; rho is a few percent of R where the field varies
// over many steps.  rho_k is an FP16 value h times 2^(b - 127), where b
// (1..254) is shared by the three components of the 32 cells x0 .. x0+31 of
// one row of one plane (x0 a multiple of 32) and held in the low byte of that
// row segment's scale word; b puts the segment's largest |rho| in [2^14,
// 2^15), so every value keeps FP16's 11 significant bits down to 2^-29 of it.
// Words are laid out [z][x / 32][y] with each segment's column padded to
// r16_rows(ny) words (TMA stages a tile's 8 rows as one 32-byte box).  An
// all-zero word decodes to 0.
__host__ __device__ inline int r16_segments(int nx) { return (nx + 31) / 32; }
__host__ __device__ inline int r16_rows(int ny) { return (ny + 7) & ~7; }
__host__ __device__ inline size_t r16_words(int nx, int ny, int nz)
{
    return (size_t)nz * r16_segments(nx) * r16_rows(ny);
}
// Compact nine-field step (d_cur == d_prev == R, updated in place) + Mur.
int launch_step_compact(const NativeConsts &c, cudaStream_t s);
int launch_h_e_compact(const NativeConsts &c, cudaStream_t s);
// The same with R in 16 bits (c.r_exp set): the step, and its first kernel.
int launch_step_compact16(const NativeConsts &c, cudaStream_t s);
int launch_h_e_compact16(const NativeConsts &c, cudaStream_t s);

// The kernels of one step in launch order, each launchable on its own (for
// per-kernel event timing).
struct StepKernel {
    const char *name;
    int (*launch)(const NativeConsts &, cudaStream_t);
};
int step_kernels(int kernel_kind, const NativeConsts &c, StepKernel *out, int max);

// H, D, sources and E of one step in the single-pass kernel (the Mur faces
// follow in launch_mur).
int launch_h_de_fused(const NativeConsts &c, cudaStream_t s);

// Tensor maps of one single-pass launch: E^n (3), H_old (3), D^n (3),
// D^{n-1} (3), E^{n-1} (3), material classes (1).  Compact form: R (3)
// after the six halo maps, then the classes; with 16-bit R the exponent
// words follow the classes.
struct FusedMaps {
    CUtensorMap m[16];
};

// Tensor maps of one strip-kernel launch (step_strip.cu, strip_unit.cuh):
// E^n (0-2), H^{n-1/2} (3-5), R or its FP16 residuals (6-8, loaded and
// stored in place), classes (9), scale words (10, 16-bit R), H^{n+1/2}
// (11-13), E^{n+1} (14-16).
struct StripMaps {
    CUtensorMap m[17];
};
static_assert(sizeof(StripMaps) % 64 == 0, "tensor maps stay 64-byte aligned in arrays");

// One solve of a batch as the batched kernels see it (device memory).  The
// solve's completed-step count n selects c[n & 1] / maps[n & 1] (smaps in a
// batch run by the strip kernel); units [unit_begin, unit_begin +
// unit_count) are its (tile x, tile y, z chunk) work items; it is skipped
// once n reaches steps_target.
struct alignas(64) BatchDesc {
    FusedMaps maps[2];
    StripMaps smaps[2];
    NativeConsts c[2];
    int zchunk, tiles_x, tiles_y, chunks;
    int unit_begin, unit_count;
    int steps_target;
    int pad;
};

// One work unit of the batched strip kernel, found by its index: the planes
// of its tile that hold no Debye memory (bit j: plane zc0 + j), its solve's
// step counter and step target, the solve, the tile (bx, by), the z chunk bz
// and the chunk length.
struct alignas(16) BatchUnit {
    unsigned long long memless;
    const int *counter;
    int solve;
    unsigned short bx, by, bz, zchunk;
    int steps_target;
};
static_assert(sizeof(BatchUnit) == 32, "two 16-byte copies per record");

// One face block of the batched Mur launch: solve, face set, first cell;
// a block of 256 threads updates BATCH_MUR_CELLS consecutive cells of the set
// (up to `limit`).
constexpr int BATCH_MUR_CELLS = 1024;
static_assert(BATCH_MUR_CELLS % 256 == 0, "whole cells per thread");
struct BatchMurBlock {
    int solve, face, first;
    int limit;  // update only the set's first `limit` cells (0: all)
};

struct BatchLaunch {
    const BatchDesc *descs;
    int nsolves;
    int total_units;
    int *work_counter;
    const BatchMurBlock *mur_blocks;
    int nmur_blocks;
    int persistent_ctas;
    int compact;      // the batch's solves keep the compact state (d_cur == d_prev == R)
    int max_classes;  // largest class count of the batch's solves (shared-memory table)
    int r16;          // the compact state holds R in 16 bits (compact is set too)
    int strip;        // compact forms: run by the strip kernel of shape strip_shape
    int strip_shape;
    const BatchUnit *units;  // strip kernel: one record per unit
};

// Tensor maps of a single-pass launch over c's buffers (false: not encodable).
bool encode_fused_maps(const NativeConsts &c, FusedMaps *maps);
bool encode_step_maps(const NativeConsts &c, bool compact, FusedMaps *maps, bool r16 = false);
int fused_tile_height();
int fused_zchunk(int nz);
int compact_zchunk(int nz);
int zchunk_limited(int nz, int max_planes);  // nz in equal chunks of at most max_planes planes
// One batched step: fused kernel over all units, Mur faces, step counters.
int launch_batch_step(const BatchLaunch &b, cudaStream_t s);
int batch_persistent_ctas(bool compact, int nclasses, bool r16 = false);
// The batch's persistent strip kernel (batch_strip.cu): its launch and the
// CTAs that fill the device at the given shape and class count.
int launch_batch_strip(const BatchLaunch &b, cudaStream_t s);
int batch_strip_ctas(bool r16, int shape, int nclasses);

// The compact forms' step kernel with TMA loads and stores over column strips
// (step_strip.cu); usable when every array is TMA-addressable (rows of a
// multiple of 16 cells, 16-byte aligned bases, R updated in place).
bool strip_usable(const NativeConsts &c, bool r16);
// Strip shapes (0 .. 3) and their tile rows; the shape a single solve runs
// (FDTD_STRIP_SHAPE overrides); the z chunk of a single solve's strip launch.
int strip_shape_rows(int shape);
int strip_single_shape(bool r16);
int strip_zchunk(int nz);
// Memoryless tile-planes (see NativeConsts::memless): strip_plane_flags marks
// each (z, 32 x 8 tile) whose cells all have classes with tau
// (specs[4 k + 3]) = 0, for a class volume of row pitch `pitch`, laid out
// [z][tile y][tile x]; strip_unit_masks packs them into one 64-bit word per
// unit of ty-row tiles (ty a multiple of 8) and z chunks of zchunk planes,
// units ordered (z chunk, tile y, tile x) with tile x fastest, and returns
// the fraction of the grid's cells on such planes.
std::vector<unsigned char> strip_plane_flags(const uint8_t *mat, int nx, int ny, int nz, int pitch, const float *specs,
                                             int nclasses);
double strip_unit_masks(const std::vector<unsigned char> &flags, int nx, int ny, int nz, int ty, int zchunk,
                        unsigned long long *masks);
int launch_strip_compact(const NativeConsts &c, cudaStream_t s);
int launch_strip_compact16(const NativeConsts &c, cudaStream_t s);

// Reads and clears the plan's device error flag (FDTD_ERR_DEVICE_TIMEOUT if set).
int plan_error(const fdtd_plan *p);

// The checks fdtd_plan_create makes of the parameters and the scheme
// (grid of at least 3 cells per axis and at most 65535 planes, sources inside
// the grid): FDTD_OK or FDTD_ERR_INVALID, before any allocation.
int plan_params_check(const FdtdParams *p, int scheme);

// fdtd_plan_create with the plan's device memory taken from pool in stream
// order on stream (copies and fills on that stream, which is synchronised
// before the call returns); with a null pool and stream, as fdtd_plan_create.  plan_destroy_on
// frees a pooled plan in stream order on stream (no device-wide wait), any
// other plan as fdtd_plan_destroy does.
int plan_create_on(const FdtdParams *p, const float *specs, int nclasses, int scheme, const float *const rp_host[6],
                   cudaMemPool_t pool, cudaStream_t stream, fdtd_plan **out);
void plan_destroy_on(fdtd_plan *plan, cudaStream_t stream);

}  // namespace fdtd
