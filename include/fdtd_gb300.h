/*
 * fdtd_gb300.h -- C ABI of libfdtd_gb300.so, a GB300-native (sm_103a)
 * implementation of the 3-D Yee FDTD time-step loop with single-pole Debye
 * media and first-order Mur boundaries of rafalgrodzinski/fdtd.
 *
 * Conventions
 *  - Every field is float32, structure of arrays, x fastest:
 *    index = z*ny*nx + y*nx + x (the reference's OFFSET macro, utils.h:15).
 *  - Device pointers are plain CUDA device addresses; streams are
 *    cudaStream_t values (fdtd_stream_t, NULL = legacy default stream).
 *  - Every entry point returns a status instead of exiting the process (the
 *    reference's CHECK macro prints and calls exit, utils.h:5-13):
 *    0 = success, 1..9999 = the cudaError_t of a failed CUDA call,
 *    >= 10000 = an FDTD_ERR_* code below.
 *  - Kernel launchers are asynchronous on the given stream; they return the
 *    launch status (cudaGetLastError), not the completion status.
 *  - Thread safety: functions that do not take an fdtd_solver may be called
 *    from any host thread; one fdtd_solver must be driven from one thread.
 */
#ifndef FDTD_GB300_H
#define FDTD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *fdtd_stream_t; /* identical to cudaStream_t */

enum fdtd_status_code {
    FDTD_OK = 0,
    FDTD_ERR_INVALID = 10001,     /* argument or size out of range */
    FDTD_ERR_IO = 10002,          /* a file could not be opened, read or written */
    FDTD_ERR_FORMAT = 10003,      /* an input file does not follow the reference format */
    FDTD_ERR_NO_SYMBOLS = 10004,  /* a compat launcher ran before fdtd_copy_symbols on this device */
    FDTD_ERR_NOMEM = 10005,       /* a host allocation failed */
    FDTD_ERR_STATE = 10006,       /* call not valid in the object's current state */
    FDTD_ERR_DEVICE_TIMEOUT = 10007, /* a kernel's bounded wait gave up; its results are invalid */
    FDTD_ERR_BUSY = 10008         /* the queued GPU work a ticket marks has not finished yet */
};

/* Human-readable text for any status this library returns. */
const char *fdtd_status_string(int status);

/* Limits shared with the reference's constant block (fdtd_calculations.h:7-8). */
#define FDTD_MAX_SOURCES 16
#define FDTD_JZ_LEN 65536          /* host source table length (fdtd.cu:1031) */
#define FDTD_MAX_CLASSES 256       /* material classes of the uint8 volume */

/* Parameter block: same members, types and order as the reference's
 * FdtdParams (fdtd.h:7-34), so a caller's struct can be passed unchanged. */
typedef struct FdtdParams {
    int nx, ny, nz;
    int iterationsCount;
    char *inputPath;
    char *outputPath;
    int elementsPerWave;
    float waveFrequency;
    float pulseWidth;
    float pulseModulationFrequency;
    int sourcesCount;
    int *sources;                  /* 3*sourcesCount ints, 0-based x, y, z */
    float defaultSigma;
    float defaultEpsS;
    float defaultEpsI;
    float defaultTauD;
    int jzCount;
    float *jz;
    float pi;
    float c;
    float timeskip;
    float lambda;
    float dt;
    float dx, dy, dz;
    float mu0;
    float eps0;
} FdtdParams;

/* ------------------------------------------------------------------------
 * Host set-up: the reference's input formats (all host memory).
 * ---------------------------------------------------------------------- */

/* Replaces initParamsWithPath (fdtd.cu:547-637): fixed line order, keys
 * ignored, t_max rounded up to a multiple of 3, sources made 0-based, and
 * c, dx = dy = dz, dt (timeskip 1.0), mu0, eps0 derived with the reference's
 * float/double mix.  inputPath, outputPath and sources are malloc'd; release
 * them with fdtd_params_free.  FDTD_ERR_FORMAT if a line does not scan. */
int fdtd_params_read(const char *path, FdtdParams *out);

/* Re-derives lambda, dx, dy, dz, dt, mu0 and eps0 with a time-step factor
 * (the reference hard-codes timeskip = 1.0, fdtd.cu:627): dt is multiplied by
 * timeskip exactly as the reference's formula does. */
int fdtd_params_set_timeskip(FdtdParams *p, float timeskip);

/* Frees the strings, the source list and the jz table of *p (replaces
 * deallocParams, fdtd.cu:640-645) and zeroes those members. */
void fdtd_params_free(FdtdParams *p);

/* Replaces setupSources (fdtd.cu:1027-1082): allocates p->jz with
 * FDTD_JZ_LEN floats and sets p->jzCount. */
int fdtd_setup_sources(FdtdParams *p);

/* Replaces setupMurBoundary (fdtd.cu:942-1024) over per-cell material arrays
 * (nx*ny*nz each).  Slab shapes: rpx0/rpxEnd 2 x ny x nz, rpy0/rpyEnd
 * nx x 2 x nz, rpz0/rpzEnd nx x ny x 2 (OFFSETRP, utils.h:16).  The reference
 * calls it before loadMaterials (fdtd.cu:59,65), i.e. on the default
 * material; pass default-filled arrays to reproduce that. */
int fdtd_setup_mur(const FdtdParams *p, const float *sigma, const float *epsS, const float *epsI,
                   const float *tauD, float *rpx0, float *rpy0, float *rpz0, float *rpxEnd,
                   float *rpyEnd, float *rpzEnd);

/* Same slabs for a volume made of one material (what the reference's call
 * order produces): every entry gets the value of (sigma, epsS, epsI, tauD). */
int fdtd_setup_mur_uniform(const FdtdParams *p, float sigma, float epsS, float epsI, float tauD,
                           float *rpx0, float *rpy0, float *rpz0, float *rpxEnd, float *rpyEnd,
                           float *rpzEnd);

/* Reads a mat_specs file as loadMaterials does (fdtd.cu:878-904): at most 94
 * records "code name sigma eps_s eps_i tau", a record that fails to scan
 * repeats the previous one, reading stops after a code >= 94.  specs receives
 * FDTD_MAX_CLASSES x 4 floats (sigma, eps_s, eps_i, tau; unlisted codes 0). */
int fdtd_read_specs(const char *specsPath, float *specs);

/* Replaces the voxel half of loadMaterials (fdtd.cu:909-936) in the native
 * form: nz slices <materialsPath>/v1_%05d.pgm (1-based), each a 6-token
 * header then nx*ny codes read as one flat stream (the header's width and
 * height are not used).  codes receives nx*ny*nz uint8 class indices.
 * Slices are parsed in parallel with nthreads host threads (0 = all cores).
 * FDTD_ERR_FORMAT on a short slice or a code outside 0..255. */
int fdtd_load_material_codes(const FdtdParams *p, const char *materialsPath, uint8_t *codes,
                             int nthreads);

/* fdtd_load_material_codes through a binary cache of the class volume (no
 * counterpart in the reference, which parses its nz text slices on every
 * run).  When cachePath holds a volume of these dimensions made from slice
 * files of the same sizes and modification times, the volume is read from
 * it; otherwise the slices are parsed and the cache is (re)written, on a
 * best-effort basis (a cache that cannot be written is not an error).
 * *fromCache (optional) receives 1 when the cache was used, else 0. */
int fdtd_load_material_codes_cached(const FdtdParams *p, const char *materialsPath, const char *cachePath,
                                    uint8_t *codes, int nthreads, int *fromCache);

/* Replaces loadMaterials (fdtd.cu:875-939) in the reference's form: four
 * per-cell float arrays looked up from the specs table. */
int fdtd_load_materials(const FdtdParams *p, const char *specsPath, const char *materialsPath,
                        float *sigma, float *epsS, float *epsI, float *tauD);

/* Replaces writeResults3d (fdtd.cu:1288-1494): for H, D, E and x, y, z one
 * text file per z plane, <outputPath>/{H|D|E}_field_{x|y|z}_%05d_z%05d.out
 * (0-based iteration, plane), ny lines of nx values " % 9.3E".  Any field
 * pointer may be NULL to skip it.  Files are formatted by nthreads host
 * threads (0 = all cores); the bytes are identical to the reference's. */
int fdtd_write_results3d(const FdtdParams *p, const float *hx, const float *hy, const float *hz,
                         const float *dx, const float *dy, const float *dz, const float *ex,
                         const float *ey, const float *ez, int iteration, int nthreads);

/* ------------------------------------------------------------------------
 * Reference-compatible kernel launchers (fdtd_calculations.h:18-42).
 * Same argument lists, roles and per-component index ranges as the
 * reference kernels; each reads the parameter block that fdtd_copy_symbols
 * stored for the current device.  Target and source buffers must not alias
 * (except as the reference itself passes them).
 * ---------------------------------------------------------------------- */

/* Replaces copySymbolsToDevice (fdtd_calculations.cu:7-29): grid size, dt,
 * dx, dy, dz, mu0, eps0, sources (FDTD_ERR_INVALID beyond FDTD_MAX_SOURCES,
 * where the reference would read past dSources) and the whole jz table (the
 * reference keeps jz[0..511] only, so its iterations >= 512 are undefined). */
int fdtd_copy_symbols(const FdtdParams *p);

/* updateHField (fdtd_calculations.cu:32-77): H -= dt/mu0 curl E^n, in place. */
int fdtd_update_h(float *hx, float *hy, float *hz, const float *exSource, const float *eySource,
                  const float *ezSource, fdtd_stream_t stream);

/* updateDField (fdtd_calculations.cu:80-122): D_target = D_source + dt curl H. */
int fdtd_update_d(float *dxTarget, float *dyTarget, float *dzTarget, const float *dxSource,
                  const float *dySource, const float *dzSource, const float *hx, const float *hy,
                  const float *hz, fdtd_stream_t stream);

/* updateEField (fdtd_calculations.cu:125-184): Debye E update from E^n
 * (Source0), E^{n-1} (Source1), D^{n+1} (dSource0), D^n, D^{n-1} and the
 * per-cell sigma, eps_inf, eps_s, tau. */
int fdtd_update_e(float *exTarget, float *eyTarget, float *ezTarget, const float *exSource0,
                  const float *eySource0, const float *ezSource0, const float *exSource1,
                  const float *eySource1, const float *ezSource1, const float *dxSource0,
                  const float *dySource0, const float *dzSource0, const float *dxSource1,
                  const float *dySource1, const float *dzSource1, const float *dxSource2,
                  const float *dySource2, const float *dzSource2, const float *sigma,
                  const float *epsI, const float *epsS, const float *tauD, fdtd_stream_t stream);

/* updateSources (fdtd_calculations.cu:187-213): Dz at each source cell =
 * Dz_source + curl - jz[currIteration].  One warp, not a full-grid launch. */
int fdtd_update_sources(float *dzTarget, const float *dzSource, const float *hx, const float *hy,
                        int currIteration, fdtd_stream_t stream);

/* updateMurBoundary (fdtd_calculations.cu:216-428): first-order Mur on the
 * tangential E of the six faces, edges excluded, including the reference's
 * ey x = nx-1 term that reads eySource at x-1 twice (:323).  Launched over
 * the face cells only. */
int fdtd_update_mur(float *exTarget, float *eyTarget, float *ezTarget, const float *exSource,
                    const float *eySource, const float *ezSource, const float *rpx0,
                    const float *rpy0, const float *rpz0, const float *rpxEnd, const float *rpyEnd,
                    const float *rpzEnd, fdtd_stream_t stream);

/* ------------------------------------------------------------------------
 * Native fused path: uint8 material classes, two E and two D slots updated
 * in place, fused kernels.  No reference counterpart; it computes the same
 * step as the five kernels above (same ranges, same order of effects).
 * ---------------------------------------------------------------------- */

/* Scheme: FDTD_SCHEME_REFERENCE reproduces the reference exactly, including
 * its E^n coefficient d = 2b - sigma dt^2 (|E| doubles every step in vacuum),
 * the ey Mur term at x = nx-1 and the source sample jz[n - n%3].
 * FDTD_SCHEME_CORRECTED uses d = a + b - sigma dt^2, the E^{n+1} term on
 * that Mur face and jz[n]. */
enum { FDTD_SCHEME_REFERENCE = 0, FDTD_SCHEME_CORRECTED = 1 };

/* Per-run constants on the device: Debye coefficients per material class,
 * sources, the jz table and the Mur slabs.  Created once, read by the native
 * kernels; immutable afterwards. */
typedef struct fdtd_plan fdtd_plan;

/* specs: nclasses x 4 floats (sigma, eps_s, eps_i, tau).  rp: the six Mur
 * slabs on the host (NULL: computed from p's default material, as the
 * reference does).  jz: p->jz if non-NULL, else built by fdtd_setup_sources. */
int fdtd_plan_create(const FdtdParams *p, const float *specs, int nclasses, int scheme,
                     const float *const rp_host[6], fdtd_plan **out);
int fdtd_plan_destroy(fdtd_plan *plan);

/* Synchronises the device and reports (then clears) the plan's error flag:
 * FDTD_ERR_DEVICE_TIMEOUT if a kernel gave up a bounded wait. */
int fdtd_plan_status(fdtd_plan *plan);

/* Device state of the native path.  E and D keep two slots each: the
 * "prev" slot holds step n-1 on entry and receives step n+1. */
typedef struct fdtd_native_fields {
    float *hx, *hy, *hz;                /* H^{n-1/2} on entry */
    float *hx_out, *hy_out, *hz_out;    /* receives H^{n+1/2} */
    float *ex, *ey, *ez;                /* E^n, read only */
    float *ex_prev, *ey_prev, *ez_prev; /* E^{n-1} in, E^{n+1} out */
    float *dx, *dy, *dz;                /* D^n, read only */
    float *dx_prev, *dy_prev, *dz_prev; /* D^{n-1} in, D^{n+1} out */
    const uint8_t *material;            /* class per cell */
} fdtd_native_fields;

/* H half step (fused three components).  hx_out may equal hx (in place). */
int fdtd_step_h(const fdtd_plan *plan, const fdtd_native_fields *f, fdtd_stream_t stream);

/* D update, sources (sample for step index n), Debye E update and the Mur
 * faces of step n.  Reads H^{n+1/2} from hx_out..hz_out. */
int fdtd_step_de(const fdtd_plan *plan, const fdtd_native_fields *f, int n, fdtd_stream_t stream);

/* Whole step n in one z-marching pass plus the Mur faces.  hx_out..hz_out
 * must not alias hx..hz (H is double-buffered). */
int fdtd_step(const fdtd_plan *plan, const fdtd_native_fields *f, int n, fdtd_stream_t stream);

/* One single-pass step (as fdtd_step) that allocates no device memory.
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * a process whose device memory belongs to another allocator (a framework's
 * caching pool, a budget fixed at start-up) or code where an allocation is
 * not allowed.  Instead of a plan it keeps the per-class Debye table, this
 * step's source sample and an error word in a file-scope __device__ array of
 * FDTD_STATIC_SCRATCH_BYTES bytes, which every GPU that loads the library
 * holds until the process exits; everything else comes from the caller:
 * p (grid, dt, dx.., sources, host jz table: required when there are
 * sources, else FDTD_ERR_INVALID; the sample of step n is jz[n] (corrected
 * scheme) or jz[n - n%3] (reference scheme) when that index is below
 * min(jzCount, FDTD_JZ_LEN), else 0, as in the plan), specs (host, nclasses x 4,
 * nclasses <= FDTD_STATIC_MAX_CLASSES, else FDTD_ERR_INVALID), the device
 * fields f (hx_out..hz_out must not alias hx..hz), the six device Mur slabs
 * rp_dev (rpx0, rpy0, rpz0, rpxEnd, rpyEnd, rpzEnd) and the step index n.
 * The first call on a device looks up the array's device address with that
 * device current; make that first call before any stream capture.  All calls
 * share the array and it keeps the last call's contents (each call rewrites
 * the table and the sample and clears the error word), so calls whose work
 * overlaps on the GPU race.  Returns after the step has finished on the GPU:
 * FDTD_OK, a CUDA error, or FDTD_ERR_DEVICE_TIMEOUT. */
#define FDTD_STATIC_MAX_CLASSES 64
#define FDTD_STATIC_SCRATCH_BYTES (FDTD_STATIC_MAX_CLASSES * 32 + 256)
int fdtd_step_static(const FdtdParams *p, const float *specs, int nclasses, int scheme,
                     const fdtd_native_fields *f, const float *const rp_dev[6], int n, fdtd_stream_t stream);

/* ------------------------------------------------------------------------
 * Solver handle: owns the device state of one solve, runs the step loop as
 * a CUDA graph and streams snapshots through pinned buffers on a side stream.
 * ---------------------------------------------------------------------- */

typedef struct fdtd_solver fdtd_solver;

enum {
    FDTD_KERNEL_SINGLE_PASS = 0,  /* fdtd_step: one z-marching kernel per step */
    FDTD_KERNEL_TWO_PASS = 1,     /* fdtd_step_h + fdtd_step_de */
    /* Single pass over nine stored fields instead of fifteen: D and E^{n-1}
     * are folded into one recursion variable per component,
     *   R^n = -a E^{n-1} - 2 tau (D^n - D^{n-1}),
     *   E^{n+1} = c (d E^n + (2 dt + 2 tau)(D^{n+1} - D^n) + R^n),
     * the same update as updateEField (fdtd_calculations.cu:141-183)
     * rearranged, 73 instead of 97 bytes of traffic per cell update.  D is not
     * stored: the D fields cannot be read, snapshotted or probed. */
    FDTD_KERNEL_COMPACT = 2,
    /* The compact form with R stored in 16 bits (no reference counterpart;
     * the reduced-storage form).  Stored per cell and component is the
     * residual rho = R^{n+1} + a E^{n+1} (a = 2 eps0 eps_inf tau), from
     * which the next step recovers R with the FP32 E it reads; rho is an
     * FP16 value times a power of two shared by the three components of
     * the 32 cells of one x-row segment of one plane (one scale per
     * segment, placing its largest residual just below 2^15, so every
     * residual keeps FP16's 11 significant bits).  H and E stay FP32 and all
     * arithmetic is FP32.  61.25
     * instead of 73 bytes of traffic per cell update.  D is not stored, as
     * in FDTD_KERNEL_COMPACT. */
    FDTD_KERNEL_COMPACT_R16 = 3
};

/* Field selectors; bit (1 << FDTD_FIELD_x) in snapshot masks. */
enum {
    FDTD_FIELD_HX = 0, FDTD_FIELD_HY, FDTD_FIELD_HZ,
    FDTD_FIELD_DX, FDTD_FIELD_DY, FDTD_FIELD_DZ,
    FDTD_FIELD_EX, FDTD_FIELD_EY, FDTD_FIELD_EZ,
    FDTD_FIELD_COUNT
};

typedef struct fdtd_solver_config {
    const FdtdParams *params;   /* grid, constants, sources, optional jz */
    const uint8_t *material;    /* host: nx*ny*nz class indices */
    const float *specs;         /* host: nclasses x 4 (sigma, eps_s, eps_i, tau) */
    int nclasses;               /* rows of specs, 1 .. FDTD_MAX_CLASSES; every class index
                                   must be below it.  The solve keeps the rows up to the
                                   largest class present in the material. */
    int scheme;                 /* FDTD_SCHEME_* */
    int kernel;                 /* FDTD_KERNEL_* */
    int device;                 /* CUDA device ordinal */
} fdtd_solver_config;

int fdtd_solver_create(const fdtd_solver_config *cfg, fdtd_solver **out);
int fdtd_solver_destroy(fdtd_solver *s);
/* Compact forms: the share of a step's cell-updates that lie on tile-planes
 * (32 x 8 cells of one z plane) whose classes all have tau = 0.  There the
 * recursion variable R stays +0, and the step kernel neither reads nor writes
 * it (no reference counterpart: the reference stores its Debye history for
 * every cell).  0 for the D form. */
double fdtd_solver_memless_fraction(const fdtd_solver *s);

/* Enqueue nsteps steps on the solver's stream (asynchronous). */
int fdtd_solver_run(fdtd_solver *s, int nsteps);
int fdtd_solver_synchronize(fdtd_solver *s);

/* Number of completed-or-enqueued steps. */
int fdtd_solver_steps(const fdtd_solver *s);

/* Test hook of the failure path (no counterpart in the reference): the next
 * single-pass step launched with TMA staging has its first CTA arm one plane's
 * barrier without issuing the copies, so that CTA's bounded wait (0.2 s) runs
 * out; the CTA raises the solver's error flag and exits, the launch completes,
 * and fdtd_solver_synchronize returns FDTD_ERR_DEVICE_TIMEOUT (once).  The
 * fields of that step are not valid afterwards; the device context is. */
int fdtd_solver_test_stall(fdtd_solver *s);

/* Copies the current value of one field (after the last enqueued step) into
 * host memory (nx*ny*nz floats); synchronises the solver first. */
int fdtd_solver_get_field(fdtd_solver *s, int field, float *host_out);

/* The solver's CUDA stream (cudaStream_t). */
fdtd_stream_t fdtd_solver_stream(const fdtd_solver *s);

/* Snapshot callback: called on a library thread with the step index (0-based,
 * the step just completed), the field id and nx*ny*nplanes floats in pinned
 * host memory that stay valid until the callback returns. */
typedef void (*fdtd_snapshot_fn)(void *user, int step, int field, const float *data, int z0, int nplanes);

/* Files written when no callback is given.  Text: the reference layout, one
 * "{H,D,E}_field_{x,y,z}_%05d_z%05d.out" file per field and plane
 * (writeResults3d, fdtd.cu:1288-1494).  Binary: one
 * "{H,D,E}_field_{x,y,z}_%05d_z%05d_n%05d.f32" file per field holding the
 * nplanes x ny x nx floats from plane z0 as they are in memory (little-endian
 * float32, x fastest): the exact values, for parity checks and fast reading
 * (no counterpart in the reference). */
enum { FDTD_SNAPSHOT_TEXT = 0, FDTD_SNAPSHOT_BINARY = 1, FDTD_SNAPSHOT_TEXT_AND_BINARY = 2 };

typedef struct fdtd_snapshot_spec {
    int every;                  /* 0 disables; else every `every` steps */
    uint32_t field_mask;        /* bits 1 << FDTD_FIELD_* */
    int z0, nplanes;            /* z range copied; nplanes 0 = whole volume */
    fdtd_snapshot_fn callback;  /* NULL: write files under output_dir */
    void *user;
    const char *output_dir;     /* used when callback is NULL */
    int writer_threads;         /* text formatting threads (0 = all cores) */
    int format;                 /* FDTD_SNAPSHOT_*, used when callback is NULL */
} fdtd_snapshot_spec;

/* Installs (or with every == 0 removes) the snapshot schedule.  Device-to-host
 * copies run on a side stream into a pinned ring and overlap the next step. */
int fdtd_solver_set_snapshots(fdtd_solver *s, const fdtd_snapshot_spec *spec);

/* Waits for every snapshot of enqueued steps to be delivered. */
int fdtd_solver_flush_snapshots(fdtd_solver *s);

/* ---- checkpoint / resume (no reference counterpart) ----
 * fdtd_solver_checkpoint writes the solve's state after the last enqueued
 * step -- H, E^n, E^{n-1}, D^n, D^{n-1} (15 float arrays), the step count and
 * a checksum of the material volume -- to a binary file.  fdtd_solver_restore
 * loads such a file into a solver created with the same configuration
 * (FDTD_ERR_FORMAT if grid, scheme or materials differ) and continues from
 * its step count; the continued run is identical to an uninterrupted one. */
int fdtd_solver_checkpoint(fdtd_solver *s, const char *path);
int fdtd_solver_restore(fdtd_solver *s, const char *path);

/* ---- on-device monitors (FP64 accumulators; no reference counterpart) ----
 * Probes: after every step, E (x, y, z components) at up to
 * FDTD_MAX_PROBES cells is appended to a device buffer of `capacity` steps.
 * fdtd_solver_get_probes copies the series out (nsteps x nprobes x 3 floats,
 * oldest first) and sets *nsteps.  Installing probes or a DFT replaces the
 * previous monitor of that kind and restarts it. */
#define FDTD_MAX_PROBES 64
int fdtd_solver_set_probes(fdtd_solver *s, int nprobes, const int *xyz, int capacity);
int fdtd_solver_get_probes(fdtd_solver *s, float *out, int *nsteps);

/* Running DFT of E at one frequency: every `stride` steps, for the planes
 * [z0, z0 + nplanes) (nplanes 0 = all), acc_c += E_c(t) exp(-i 2 pi f t) *
 * stride * dt in double precision, t = (steps completed) * dt. */
int fdtd_solver_set_dft(fdtd_solver *s, double frequency, int stride, int z0, int nplanes);
/* Copies the accumulators of component comp (0 x, 1 y, 2 z) as
 * nx*ny*nplanes doubles each (re, im; either may be NULL). */
int fdtd_solver_get_dft(fdtd_solver *s, int comp, double *re, double *im);
/* Spectral SAR from the DFT accumulators: sigma(class) |E_f|^2 / (2 rho(class))
 * per cell, reduced on the device to its maximum (*peak) and that cell's
 * linear index (*cell).  rho: nclasses densities in kg/m^3 (NULL: 1000 for
 * every class). */
int fdtd_solver_peak_sar(fdtd_solver *s, const float *rho, double *peak, long long *cell);

/* Kernel timing (the role of the reference's nvprof job scripts,
 * run_fdtd_prof*-rafal.sh): runs nsteps steps launching each kernel directly,
 * bracketed by CUDA events on the solver stream, and returns the average
 * duration in milliseconds of each of the step's kernels in launch order
 * (at most max_kernels; *nkernels receives the count).  The steps advance
 * the solve like fdtd_solver_run. */
int fdtd_solver_profile(fdtd_solver *s, int nsteps, float *avg_ms, int max_kernels, int *nkernels);

/* Name of kernel k of a step, as reported by fdtd_solver_profile. */
const char *fdtd_solver_kernel_name(const fdtd_solver *s, int k);

/* ------------------------------------------------------------------------
 * Batch: many independent solves of uneven sizes advanced together (no
 * reference counterpart).  Each solve keeps its own resident state and plan;
 * one batched step is one kernel over the column-tile x z-chunk work units of
 * every solve (compact forms: one CTA per unit; D form: persistent CTAs taking
 * units from a counter), one Mur launch over every solve's face cells and a
 * counter advance, replayed as a CUDA graph.  A solve stops at its own step
 * target; adding or removing a solve rebuilds the launch.  Results of a solve
 * are identical whether it runs alone or with others.
 *
 * A running batch is never drained for bookkeeping: fdtd_batch_add uploads
 * the new solve on a side stream (the batch stream waits for it before the
 * solve's first step), fdtd_batch_remove frees in stream order behind the
 * steps already queued, and fdtd_batch_read_async / fdtd_batch_mark queue a
 * copy or a marker and return a ticket that fdtd_batch_ticket polls.  Device
 * memory of the solves comes from the batch's own stream-ordered pool, which
 * keeps freed memory for later solves until the batch is destroyed.
 * ---------------------------------------------------------------------- */

typedef struct fdtd_batch fdtd_batch;

/* A batch of the D form (FDTD_KERNEL_SINGLE_PASS state: every field readable). */
int fdtd_batch_create(int device, fdtd_batch **out);
/* A batch whose solves all keep the state of `kernel`: FDTD_KERNEL_SINGLE_PASS
 * (D form), FDTD_KERNEL_COMPACT (nine fields, D not readable) or
 * FDTD_KERNEL_COMPACT_R16 (the same with R in 16 bits). */
int fdtd_batch_create_form(int device, int kernel, fdtd_batch **out);
int fdtd_batch_destroy(fdtd_batch *b);
/* Device bytes one D-form solve of this grid needs (state + plan), for admission. */
size_t fdtd_batch_solve_bytes(int nx, int ny, int nz);
/* The same for a solve of this batch's form. */
size_t fdtd_batch_need_bytes(const fdtd_batch *b, int nx, int ny, int nz);
/* Adds a solve (cfg->kernel and cfg->device are ignored: the batch's form and
 * device apply) that will run `steps` steps; *id receives its handle.  Waits
 * only for the solve's own uploads, not for queued steps; it joins at the
 * next fdtd_batch_run. */
int fdtd_batch_add(fdtd_batch *b, const fdtd_solver_config *cfg, int steps, int *id);
/* Removes a solve; its memory is released in stream order after the steps
 * and reads already queued (no wait). */
int fdtd_batch_remove(fdtd_batch *b, int id);
/* Enqueues nsteps batched steps (asynchronous). */
int fdtd_batch_run(fdtd_batch *b, int nsteps);
/* Chooses the z-blocking depth of the batched kernel for the current solves
 * and, in the compact forms, the strip kernel's tile shape (no counterpart in
 * the reference): times steps_per_trial steps (rounded up to a multiple of 8,
 * after 8 untimed steps) at each candidate (compact forms: every strip tile
 * shape and the z-marching kernel, with largest z chunks of 8, 16, 32, 64
 * planes; D form 16-64 planes) and
 * keeps the one with the least time per cell-update.  The trial steps are real steps of the solves
 * (a cell's update does not depend on where chunks meet, so the results are
 * the same bits).  *chosen (optional): the chunk limit kept, 0 if no trial
 * advanced a solve (the form's default stays).  Synchronises. */
int fdtd_batch_autotune(fdtd_batch *b, int steps_per_trial, int *chosen);
/* The launch shape in use (no counterpart in the reference): the largest z
 * chunk (0: the form's default), the rows of the column tiles, and for the
 * compact forms the strip kernel's shape (0-3: 2 x 4, 1 x 8 and 4 x 2 cells
 * per thread x warps on 8-row tiles, 4 x 4 on 16-row tiles; -1 for the
 * z-marching kernel and for the D form).  fdtd_batch_autotune chooses the
 * compact forms' kernel and shape together with the chunk limit, timing every
 * pair. */
int fdtd_batch_tuning(const fdtd_batch *b, int *zchunk_max, int *tile_rows, int *strip_shape);
int fdtd_batch_synchronize(fdtd_batch *b);
/* Completed steps of one solve (synchronises; -1 on error). */
int fdtd_batch_steps(fdtd_batch *b, int id);
/* Copies planes [z0, z0 + nplanes) (nplanes 0 = all) of one field of one
 * solve into host memory, nx*ny*nplanes floats. */
int fdtd_batch_get_field(fdtd_batch *b, int id, int field, int z0, int nplanes, float *host_out);
/* Queues a copy of planes [z0, z0 + nplanes) (nplanes 0 = all) of one field
 * of one solve, as they will be after the steps queued so far, into host
 * memory (nx*ny*nplanes floats; page-locked memory, e.g. fdtd_host_alloc,
 * keeps the copy asynchronous), without waiting.  *ticket: poll it with
 * fdtd_batch_ticket; host_out holds the planes once it reports done.  The
 * reference's snapshot path copies into pinned buffers the same way
 * (fdtd.cu:134-136). */
int fdtd_batch_read_async(fdtd_batch *b, int id, int field, int z0, int nplanes, float *host_out,
                          long long *ticket);
/* A ticket for the point after everything queued so far. */
int fdtd_batch_mark(fdtd_batch *b, long long *ticket);
/* FDTD_OK once the ticket's work has finished (the ticket is then spent),
 * FDTD_ERR_BUSY while it has not (wait = 0), or a CUDA error; wait != 0
 * blocks until it finishes. */
int fdtd_batch_ticket(fdtd_batch *b, long long ticket, int wait);
/* With timing on, every fdtd_batch_run is bracketed by events;
 * fdtd_batch_busy returns the GPU time of the finished runs and the time from
 * the first run's start to the last finished run's end (their ratio is the
 * fraction of time the batch kept the GPU busy). */
int fdtd_batch_set_timing(fdtd_batch *b, int on);
int fdtd_batch_busy(fdtd_batch *b, double *busy_ms, double *span_ms);
size_t fdtd_batch_bytes(const fdtd_batch *b);
int fdtd_batch_size(const fdtd_batch *b);
fdtd_stream_t fdtd_batch_stream(const fdtd_batch *b);

/* Page-locked host memory for asynchronous copies (cudaHostAlloc / cudaFreeHost). */
int fdtd_host_alloc(size_t bytes, void **out);
int fdtd_host_free(void *p);

#ifdef __cplusplus
}
#endif

#endif /* FDTD_GB300_H */
