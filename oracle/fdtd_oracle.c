/*
 * fdtd_oracle.c -- CPU restatement of the reference FDTD time-step loop.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py may load this library, and only as the checker or
 * as the timed CPU baseline -- never as part of the product path.
 *
 * One source, two builds:
 *   ORACLE_REAL=double  -> FP64 oracle (accuracy reference for every form);
 *   ORACLE_REAL=float   -> FP32 port.  Every expression keeps the operand
 *                          types of the reference (float fields, double
 *                          literals), so with -ffp-contract=off it reproduces
 *                          the reference kernels run on a CPU bit for bit.
 *
 * Reference semantics restated here (file:line within rafalgrodzinski/fdtd):
 *   updateHField        fdtd_calculations.cu:32-77
 *   updateDField        fdtd_calculations.cu:80-122
 *   updateEField        fdtd_calculations.cu:125-184
 *   updateSources       fdtd_calculations.cu:187-213
 *   updateMurBoundary   fdtd_calculations.cu:216-428
 *   slot rotation       fdtd.cu:115-530 (three E and three D slots, H in place,
 *                       source sample jz[i - i%3])
 *   initParamsWithPath  fdtd.cu:547-637
 *   loadMaterials       fdtd.cu:875-939
 *   setupMurBoundary    fdtd.cu:942-1024 (C99 complex arithmetic)
 *   setupSources        fdtd.cu:1027-1082
 *   writeResults3d      fdtd.cu:1288-1494
 *
 * The "corrected" scheme (cfg->corrected != 0) is not in the reference: it
 * replaces the E^n coefficient d = 2b - s dt^2 by d = a + b - s dt^2 (the
 * reference's d makes |E| double every step in vacuum), lets the ey Mur face
 * at x = nx-1 read E^{n+1} at x-1 like every other face, and injects the
 * source sample jz[i] at step i instead of jz[i - i%3].
 */
#include <complex.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORACLE_REAL
#define ORACLE_REAL double
#endif
typedef ORACLE_REAL real;

/* sqrt at the precision of the operand: the reference calls sqrt() on a float
 * inside device code, which selects the float overload. */
#define RSQRT(v) _Generic((v), float: sqrtf, default: sqrt)(v)

#define ORACLE_MAX_SOURCES 64
#define ORACLE_JZ_LEN (1 << 16)
#define ORACLE_SPEC_CODES 256

typedef struct {
    int nx, ny, nz;
    int iterations;                 /* rounded up to a multiple of 3 */
    char input_path[1024];
    char output_path[1024];
    int elements_per_wave;
    float wave_frequency;
    float pulse_width;
    float pulse_modulation_frequency;
    int nsources;
    int sources[3 * ORACLE_MAX_SOURCES]; /* 0-based x, y, z */
    float default_sigma, default_eps_s, default_eps_i, default_tau_d;
    float pi, c, timeskip, lambda, dt, dx, dy, dz, mu0, eps0;
} oracle_params;

typedef struct {
    int nx, ny, nz;
    float dt, dx, dy, dz, mu0, eps0;
    int nsources;
    const int *sources;   /* 3 * nsources, 0-based */
    const float *jz;      /* source table */
    int njz;
    int corrected;        /* 0: reference semantics */
    int nthreads;         /* OpenMP threads, <= 0: library default */
} oracle_cfg;

/* Reference state: H, three E slots, three D slots (fdtd.h:37-54). */
typedef struct {
    real *hx, *hy, *hz;
    real *e[3][3];        /* [slot][component] */
    real *d[3][3];
} oracle_state;

/* Per-cell material arrays and Mur slabs (float in the reference). */
typedef struct {
    const float *sigma, *eps_i, *eps_s, *tau_d;
    const float *rpx0, *rpy0, *rpz0, *rpx_end, *rpy_end, *rpz_end;
} oracle_media;

#define AT(p, x, y, z) ((p)[((size_t)(z) * (size_t)ny + (size_t)(y)) * (size_t)nx + (size_t)(x)])
/* Mur slab index: OFFSETRP with per-face (rpnx, rpny), utils.h:16 */
#define RPX(p, l, y, z) ((p)[((size_t)(z) * (size_t)ny + (size_t)(y)) * 2 + (size_t)(l)])
#define RPY(p, x, l, z) ((p)[((size_t)(z) * 2 + (size_t)(l)) * (size_t)nx + (size_t)(x)])
#define RPZ(p, x, y, l) ((p)[((size_t)(l) * (size_t)ny + (size_t)(y)) * (size_t)nx + (size_t)(x)])

static void set_threads(const oracle_cfg *cfg)
{
#ifdef _OPENMP
    if (cfg->nthreads > 0)
        omp_set_num_threads(cfg->nthreads);
#else
    (void)cfg;
#endif
}

/* H <- H - dt/mu0 curl E, in place (fdtd_calculations.cu:32-77).  The hx
 * z-derivative is scaled by dy, as in the reference (:51).  Work is shared
 * over (z, y) rows so that every host thread has rows even on thin slabs. */
static void update_h(const oracle_cfg *cfg, real *hx, real *hy, real *hz,
                     const real *ex, const real *ey, const real *ez)
{
    const int nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
    const real dt = cfg->dt, mu0 = cfg->mu0;
    const real kx = dt / (mu0 * (real)cfg->dx);
    const real ky = dt / (mu0 * (real)cfg->dy);
    const real kz = dt / (mu0 * (real)cfg->dz);
    /* hx: y in [0,ny-2]; hy: y in [1,ny-2]; hz: y in [0,ny-2], z >= 1 */
    #pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < nz - 1; z++) {
        for (int y = 0; y < ny - 1; y++) {
            for (int x = 1; x < nx - 1; x++)
                AT(hx, x, y, z) = AT(hx, x, y, z) - ky * (AT(ez, x, y + 1, z) - AT(ez, x, y, z))
                                                  + ky * (AT(ey, x, y, z + 1) - AT(ey, x, y, z));
            if (y >= 1)
                for (int x = 0; x < nx - 1; x++)
                    AT(hy, x, y, z) = AT(hy, x, y, z) - kz * (AT(ex, x, y, z + 1) - AT(ex, x, y, z))
                                                      + kx * (AT(ez, x + 1, y, z) - AT(ez, x, y, z));
            if (z >= 1)
                for (int x = 0; x < nx - 1; x++)
                    AT(hz, x, y, z) = AT(hz, x, y, z) - kx * (AT(ey, x + 1, y, z) - AT(ey, x, y, z))
                                                      + ky * (AT(ex, x, y + 1, z) - AT(ex, x, y, z));
        }
    }
}

/* D^{n+1} = D^n + dt curl H into a separate slot (fdtd_calculations.cu:80-122),
 * then the soft sources overwrite Dz at their cells (:187-213). */
static void update_d(const oracle_cfg *cfg, real *const dt_[3], real *const ds[3],
                     const real *hx, const real *hy, const real *hz, int jz_index)
{
    const int nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
    const real tx = (real)cfg->dt / (real)cfg->dx;
    const real ty = (real)cfg->dt / (real)cfg->dy;
    const real tz = (real)cfg->dt / (real)cfg->dz;
    real *dxT = dt_[0], *dyT = dt_[1], *dzT = dt_[2];
    const real *dxS = ds[0], *dyS = ds[1], *dzS = ds[2];
    /* dx: y, z in [1,n-2]; dy: y in [0,ny-2], z in [1,nz-2]; dz: y in [1,ny-2], z in [0,nz-2] */
    #pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < nz - 1; z++) {
        for (int y = 0; y < ny - 1; y++) {
            if (z >= 1 && y >= 1)
                for (int x = 0; x < nx - 1; x++)
                    AT(dxT, x, y, z) = AT(dxS, x, y, z) + ty * (AT(hz, x, y, z) - AT(hz, x, y - 1, z))
                                                        - tz * (AT(hy, x, y, z) - AT(hy, x, y, z - 1));
            if (z >= 1)
                for (int x = 1; x < nx - 1; x++)
                    AT(dyT, x, y, z) = AT(dyS, x, y, z) + tz * (AT(hx, x, y, z) - AT(hx, x, y, z - 1))
                                                        - tx * (AT(hz, x, y, z) - AT(hz, x - 1, y, z));
            if (y >= 1)
                for (int x = 1; x < nx - 1; x++)
                    AT(dzT, x, y, z) = AT(dzS, x, y, z) + tx * (AT(hy, x, y, z) - AT(hy, x - 1, y, z))
                                                        - ty * (AT(hx, x, y, z) - AT(hx, x, y - 1, z));
        }
    }
    /* updateSources: the device table holds jz[0..511]; larger indices are
     * undefined in the reference, here they read the host table. */
    const real jz = (jz_index >= 0 && jz_index < cfg->njz) ? (real)cfg->jz[jz_index] : (real)0;
    for (int s = 0; s < cfg->nsources; s++) {
        const int x = cfg->sources[3 * s], y = cfg->sources[3 * s + 1], z = cfg->sources[3 * s + 2];
        real val = AT(dzS, x, y, z) + (real)cfg->dt / (real)cfg->dx * (AT(hy, x, y, z) - AT(hy, x - 1, y, z))
                                    - (real)cfg->dt / (real)cfg->dy * (AT(hx, x, y, z) - AT(hx, x, y - 1, z))
                                    - jz;
        AT(dzT, x, y, z) = val;
    }
}

/* Debye E update (fdtd_calculations.cu:125-184).  Coefficients per cell with
 * the reference's double literals; ex over [0,nx-2]x[1,ny-2]x[1,nz-2], ey and
 * ez over the inclusive ranges [1,nx-1]x[0,ny-1]x[1,nz-1]. */
static void update_e(const oracle_cfg *cfg, const oracle_media *m,
                     real *const eT[3], real *const e0[3], real *const e1[3],
                     real *const d0[3], real *const d1[3], real *const d2[3])
{
    const int nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
    const real dt = cfg->dt, eps0 = cfg->eps0;
    const int corrected = cfg->corrected;
    #pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < nz; z++) {
        for (int y = 0; y < ny; y++) {
            for (int x = 0; x < nx; x++) {
                const int ex_on = x <= nx - 2 && y >= 1 && y <= ny - 2 && z >= 1 && z <= nz - 2;
                const int eyz_on = x >= 1 && z >= 1;
                if (!ex_on && !eyz_on)
                    continue;
                const size_t i = ((size_t)z * ny + y) * nx + x;
                const real sigma = m->sigma[i], eps_i = m->eps_i[i], eps_s = m->eps_s[i], tau = m->tau_d[i];
                real a = 2.0 * eps0 * eps_i * tau;
                real b = a + 2.0 * dt * (eps0 * eps_s + sigma * tau);
                real c = 1.0 / (b + sigma * dt * dt);
                real d = corrected ? (1.0 * a + b - sigma * dt * dt) : (2.0 * b - sigma * dt * dt);
                for (int k = 0; k < 3; k++) {
                    if (k == 0 ? !ex_on : !eyz_on)
                        continue;
                    eT[k][i] = c * (d * e0[k][i] - a * e1[k][i]
                                    + (2.0 * (dt + tau)) * d0[k][i]
                                    - (2.0 * dt + 4.0 * tau) * d1[k][i]
                                    + (2.0 * tau) * d2[k][i]);
                }
            }
        }
    }
}

/* First-order Mur value for one face cell.  rp_self is the slab layer on the
 * face, rp_nbr the layer one cell inwards; t_nbr is E^{n+1} and s_nbr, s_self
 * are E^n (fdtd_calculations.cu:240-248 and its mirrors). */
static inline real mur_cell(real dt, real h, real mu0eps0, real rp_self, real rp_nbr,
                            real t_nbr, real s_nbr, real s_self)
{
    return 1 / (dt + h * RSQRT(mu0eps0 * rp_self)) *
           ((dt - h * RSQRT(mu0eps0 * rp_nbr)) * t_nbr +
            (dt + h * RSQRT(mu0eps0 * rp_nbr)) * s_nbr -
            (dt - h * RSQRT(mu0eps0 * rp_self)) * s_self);
}

/* updateMurBoundary (fdtd_calculations.cu:216-428): tangential E on the six
 * faces, edges excluded.  With every dimension >= 3 no face reads a cell that
 * another face writes, so the face order does not matter, and the cells of
 * one face loop are independent (each loop is shared over host threads). */
static void update_mur(const oracle_cfg *cfg, const oracle_media *m,
                       real *const eT[3], real *const eS[3])
{
    const int nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
    const real dt = cfg->dt, hx_ = cfg->dx, hy_ = cfg->dy, hz_ = cfg->dz;
    const real me = (real)cfg->mu0 * (real)cfg->eps0;
    real *exT = eT[0], *eyT = eT[1], *ezT = eT[2];
    const real *exS = eS[0], *eyS = eS[1], *ezS = eS[2];
    const int fix = cfg->corrected;

    /* ex on y faces (rpy) and z faces (rpz) */
    #pragma omp parallel for schedule(static)
    for (int z = 1; z < nz - 1; z++)
        for (int x = 0; x < nx - 1; x++) {
            AT(exT, x, 0, z) = mur_cell(dt, hy_, me, RPY(m->rpy0, x, 0, z), RPY(m->rpy0, x, 1, z),
                                        AT(exT, x, 1, z), AT(exS, x, 1, z), AT(exS, x, 0, z));
            AT(exT, x, ny - 1, z) = mur_cell(dt, hy_, me, RPY(m->rpy_end, x, 1, z), RPY(m->rpy_end, x, 0, z),
                                             AT(exT, x, ny - 2, z), AT(exS, x, ny - 2, z), AT(exS, x, ny - 1, z));
        }
    #pragma omp parallel for schedule(static)
    for (int y = 1; y < ny - 1; y++)
        for (int x = 0; x < nx - 1; x++) {
            AT(exT, x, y, 0) = mur_cell(dt, hz_, me, RPZ(m->rpz0, x, y, 0), RPZ(m->rpz0, x, y, 1),
                                        AT(exT, x, y, 1), AT(exS, x, y, 1), AT(exS, x, y, 0));
            AT(exT, x, y, nz - 1) = mur_cell(dt, hz_, me, RPZ(m->rpz_end, x, y, 1), RPZ(m->rpz_end, x, y, 0),
                                             AT(exT, x, y, nz - 2), AT(exS, x, y, nz - 2), AT(exS, x, y, nz - 1));
        }
    /* ey on x faces (rpx) and z faces (rpz).  At x = nx-1 the reference reads
     * E^n at x-1 in the first term as well (fdtd_calculations.cu:323). */
    #pragma omp parallel for schedule(static)
    for (int z = 1; z < nz - 1; z++)
        for (int y = 0; y < ny - 1; y++) {
            AT(eyT, 0, y, z) = mur_cell(dt, hx_, me, RPX(m->rpx0, 0, y, z), RPX(m->rpx0, 1, y, z),
                                        AT(eyT, 1, y, z), AT(eyS, 1, y, z), AT(eyS, 0, y, z));
            const real first = fix ? AT(eyT, nx - 2, y, z) : AT(eyS, nx - 2, y, z);
            AT(eyT, nx - 1, y, z) = mur_cell(dt, hx_, me, RPX(m->rpx_end, 1, y, z), RPX(m->rpx_end, 0, y, z),
                                             first, AT(eyS, nx - 2, y, z), AT(eyS, nx - 1, y, z));
        }
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < ny - 1; y++)
        for (int x = 1; x < nx - 1; x++) {
            AT(eyT, x, y, 0) = mur_cell(dt, hz_, me, RPZ(m->rpz0, x, y, 0), RPZ(m->rpz0, x, y, 1),
                                        AT(eyT, x, y, 1), AT(eyS, x, y, 1), AT(eyS, x, y, 0));
            AT(eyT, x, y, nz - 1) = mur_cell(dt, hz_, me, RPZ(m->rpz_end, x, y, 1), RPZ(m->rpz_end, x, y, 0),
                                             AT(eyT, x, y, nz - 2), AT(eyS, x, y, nz - 2), AT(eyS, x, y, nz - 1));
        }
    /* ez on x faces (rpx) and y faces (rpy) */
    #pragma omp parallel for schedule(static)
    for (int z = 0; z < nz - 1; z++)
        for (int y = 1; y < ny - 1; y++) {
            AT(ezT, 0, y, z) = mur_cell(dt, hx_, me, RPX(m->rpx0, 0, y, z), RPX(m->rpx0, 1, y, z),
                                        AT(ezT, 1, y, z), AT(ezS, 1, y, z), AT(ezS, 0, y, z));
            AT(ezT, nx - 1, y, z) = mur_cell(dt, hx_, me, RPX(m->rpx_end, 1, y, z), RPX(m->rpx_end, 0, y, z),
                                             AT(ezT, nx - 2, y, z), AT(ezS, nx - 2, y, z), AT(ezS, nx - 1, y, z));
        }
    #pragma omp parallel for schedule(static)
    for (int z = 0; z < nz - 1; z++)
        for (int x = 1; x < nx - 1; x++) {
            AT(ezT, x, 0, z) = mur_cell(dt, hy_, me, RPY(m->rpy0, x, 0, z), RPY(m->rpy0, x, 1, z),
                                        AT(ezT, x, 1, z), AT(ezS, x, 1, z), AT(ezS, x, 0, z));
            AT(ezT, x, ny - 1, z) = mur_cell(dt, hy_, me, RPY(m->rpy_end, x, 1, z), RPY(m->rpy_end, x, 0, z),
                                             AT(ezT, x, ny - 2, z), AT(ezS, x, ny - 2, z), AT(ezS, x, ny - 1, z));
        }
}

/* Run steps [step0, step0 + nsteps) of the reference loop (fdtd.cu:115-530):
 * step i writes E and D slot i%3, reads E^n/D^n from slot (i+2)%3 and
 * E^{n-1}/D^{n-1} from slot (i+1)%3, and injects jz[i - i%3]. */
int oracle_run(const oracle_cfg *cfg, const oracle_media *m, oracle_state *s, int step0, int nsteps)
{
    if (cfg->nx < 3 || cfg->ny < 3 || cfg->nz < 3)
        return -1;
    for (int k = 0; k < cfg->nsources; k++) {
        const int *p = cfg->sources + 3 * k;
        if (p[0] < 1 || p[1] < 1 || p[2] < 0 || p[0] >= cfg->nx || p[1] >= cfg->ny || p[2] >= cfg->nz)
            return -2;
    }
    set_threads(cfg);
    for (int i = step0; i < step0 + nsteps; i++) {
        const int t = i % 3, n0 = (i + 2) % 3, n1 = (i + 1) % 3;
        update_h(cfg, s->hx, s->hy, s->hz, s->e[n0][0], s->e[n0][1], s->e[n0][2]);
        update_d(cfg, s->d[t], s->d[n0], s->hx, s->hy, s->hz, cfg->corrected ? i : i - i % 3);
        update_e(cfg, m, s->e[t], s->e[n0], s->e[n1], s->d[t], s->d[n0], s->d[n1]);
        update_mur(cfg, m, s->e[t], s->e[n0]);
    }
    return 0;
}

/* Single-kernel entry points for unit tests of each reference kernel. */
int oracle_update_h(const oracle_cfg *cfg, real *h[3], real *e[3])
{
    set_threads(cfg);
    update_h(cfg, h[0], h[1], h[2], e[0], e[1], e[2]);
    return 0;
}

int oracle_update_d(const oracle_cfg *cfg, real *dT[3], real *dS[3], real *h[3], int jz_index)
{
    set_threads(cfg);
    update_d(cfg, dT, dS, h[0], h[1], h[2], jz_index);
    return 0;
}

int oracle_update_e(const oracle_cfg *cfg, const oracle_media *m, real *eT[3], real *e0[3], real *e1[3],
                    real *d0[3], real *d1[3], real *d2[3])
{
    set_threads(cfg);
    update_e(cfg, m, eT, e0, e1, d0, d1, d2);
    return 0;
}

int oracle_update_mur(const oracle_cfg *cfg, const oracle_media *m, real *eT[3], real *eS[3])
{
    update_mur(cfg, m, eT, eS);
    return 0;
}

int oracle_real_size(void) { return (int)sizeof(real); }

/* Host threads the loops above run on for cfg (nthreads <= 0: the OpenMP
 * default, i.e. every core the process may use). */
int oracle_threads(const oracle_cfg *cfg)
{
#ifdef _OPENMP
    set_threads(cfg);
    return omp_get_max_threads();
#else
    (void)cfg;
    return 1;
#endif
}

/* ------------------------------------------------------------------ setup */

/* initParamsWithPath (fdtd.cu:547-637): fixed line order, keys ignored. */
int oracle_params_read(const char *path, oracle_params *p)
{
    char tmp[1024];
    memset(p, 0, sizeof(*p));
    FILE *f = fopen(path, "r");
    if (!f)
        return -1;
    int ok = 1;
    ok &= fscanf(f, "%1023s %d %d %d\n", tmp, &p->nx, &p->ny, &p->nz) == 4;
    ok &= fscanf(f, "%1023s %d\n", tmp, &p->iterations) == 2;
    p->iterations = ((p->iterations - 1) / 3 + 1) * 3;
    ok &= fgets(tmp, sizeof tmp, f) != NULL;                          /* nf */
    ok &= fscanf(f, "%1023s %1023s\n", tmp, p->input_path) == 2;
    ok &= fgets(tmp, sizeof tmp, f) != NULL;                          /* env_file_prefix */
    ok &= fscanf(f, "%1023s %1023s\n", tmp, p->output_path) == 2;
    for (int k = 0; k < 9; k++)                                       /* output_format .. source_type */
        ok &= fgets(tmp, sizeof tmp, f) != NULL;
    ok &= fscanf(f, "%1023s %d\n", tmp, &p->elements_per_wave) == 2;
    ok &= fscanf(f, "%1023s %g\n", tmp, &p->wave_frequency) == 2;
    ok &= fscanf(f, "%1023s %g\n", tmp, &p->pulse_width) == 2;
    ok &= fscanf(f, "%1023s %g\n", tmp, &p->pulse_modulation_frequency) == 2;
    ok &= fscanf(f, "%1023s %d\n", tmp, &p->nsources) == 2;
    if (!ok || p->nsources < 0 || p->nsources > ORACLE_MAX_SOURCES) {
        fclose(f);
        return -2;
    }
    for (int k = 0; k < p->nsources; k++) {
        int *s = p->sources + 3 * k;
        ok &= fscanf(f, "%1023s %d %d %d\n", tmp, s, s + 1, s + 2) == 4;
        s[0] -= 1;
        s[1] -= 1;
        s[2] -= 1;
    }
    ok &= fgets(tmp, sizeof tmp, f) != NULL;                          /* pulse_type */
    ok &= fscanf(f, "%1023s %f\n", tmp, &p->default_sigma) == 2;
    ok &= fscanf(f, "%1023s %f\n", tmp, &p->default_eps_s) == 2;
    ok &= fscanf(f, "%1023s %f\n", tmp, &p->default_eps_i) == 2;
    ok &= fscanf(f, "%1023s %f\n", tmp, &p->default_tau_d) == 2;
    fclose(f);
    if (!ok)
        return -3;

    /* derived constants: double expressions stored into float fields */
    p->pi = acos(-1.0);
    p->c = 3.0 * pow(10.0, 8.0);
    p->timeskip = 1.0;
    p->lambda = p->c / p->wave_frequency;
    p->dx = p->lambda / p->elements_per_wave;
    p->dy = p->dx;
    p->dz = p->dx;
    p->dt = 1.0 * p->timeskip /
            (p->c * sqrt(1.0 / pow(p->dx, 2.0) + 1.0 / pow(p->dy, 2.0) + 1.0 / pow(p->dz, 2.0)));
    p->mu0 = 4.0 * p->pi * pow(10.0, -7.0);
    p->eps0 = 1.0 / (p->mu0 * p->c * p->c);
    return 0;
}

/* dt for a Courant factor other than the reference's fixed timeskip = 1.0
 * (fdtd.cu:629-631 with timeskip as given; used for the 0.99 CFL step of the
 * benchmark configurations). */
int oracle_params_set_timeskip(oracle_params *p, float timeskip)
{
    if (!(timeskip > 0.0f) || p->elements_per_wave <= 0 || !(p->wave_frequency > 0.0f))
        return -1;
    p->timeskip = timeskip;
    p->dt = 1.0 * p->timeskip /
            (p->c * sqrt(1.0 / pow(p->dx, 2.0) + 1.0 / pow(p->dy, 2.0) + 1.0 / pow(p->dz, 2.0)));
    return 0;
}

/* setupSources (fdtd.cu:1027-1082): a sub-sampled, cosine-modulated Gaussian,
 * scaled by 1e-15/dt/3, then centrally differenced and divided by dx*dy.
 * jz receives ORACLE_JZ_LEN floats. */
int oracle_setup_sources(const oracle_params *p, float *jz)
{
    const int off = ORACLE_JZ_LEN;
    float *g = calloc((size_t)off * 2, sizeof(float));
    float *g2 = calloc((size_t)off * 2, sizeof(float));
    if (!g || !g2) {
        free(g);
        free(g2);
        return -1;
    }
    memset(jz, 0, sizeof(float) * (size_t)off);
    const int fine = (1 << 13) * p->pulse_width * p->wave_frequency * p->dt;
    const int half = 1.0 / (p->pulse_width * p->wave_frequency) / (p->dt / fine) / 2.0;
    if (fine <= 0 || half + 2 >= off) {
        free(g);
        free(g2);
        return -2;
    }
    for (int i = -half - 1; i <= half + 1; i++) {
        float v1 = ((float)i / (((float)half + 1.0) / 4.0));
        float v2 = exp(-pow(v1, 2.0));
        float v3 = cos(2.0 * acos(-1.0) * p->pulse_modulation_frequency * p->wave_frequency * i * (p->dt / fine));
        g[i + off] = v2 * v3;
    }
    int start = 0, found = 0;
    for (int i = -(1 << 12); i < (1 << 12); i++)
        if (fabs(g[i + off]) >= 1e-9 && i % fine == 0) {
            start = i;
            found = 1;
            break;
        }
    if (!found) {
        free(g);
        free(g2);
        return -3;
    }
    int n = 0;
    for (int i = start; i <= half + 1; i += fine) {
        float val = g[i + off] * 1e-15 / p->dt / 3.0;
        jz[n++] = val;
    }
    for (int i = 2; i <= (1 << 14); i++) {
        float val = (((jz[i] - jz[i - 1]) / p->dt) + ((jz[i - 1] - jz[i - 2]) / p->dt)) / 2.0 *
                    (p->dt * p->dz) / (p->dx * p->dy * p->dz);
        g2[i - 1 + off] = val;
    }
    for (int i = 0; i < (1 << 14); i++)
        jz[i] = g2[i + off + 1];
    free(g);
    free(g2);
    return 0;
}

/* One Mur slab entry: Re(eps_i + (eps_s - eps_i)/(1 + c1) - c2) with C99
 * complex operands (fdtd.cu:959-963 and mirrors); imaginary != 0 selects the
 * i-scaled c1, c2 of the y and z slabs. */
static float rp_value(const oracle_params *p, float sigma, float eps_s, float eps_i, float tau, int imaginary)
{
    float complex c1, c2;
    if (imaginary) {
        c1 = 0.0 + 2.0 * p->pi * p->wave_frequency * tau * I;
        c2 = 0.0 + sigma / (2.0 * p->pi * p->wave_frequency * p->eps0) * I;
    } else {
        c1 = 0.0 + 2.0 * p->pi * p->wave_frequency * tau;
        c2 = 0.0 + sigma / (2.0 * p->pi * p->wave_frequency * p->eps0);
    }
    return creal(eps_i + (eps_s - eps_i) / (1.0 + c1) - c2);
}

/* setupMurBoundary (fdtd.cu:942-1024) over per-cell float material arrays.
 * rpx: 2 x ny x nz, rpy: nx x 2 x nz, rpz: nx x ny x 2. */
int oracle_setup_mur(const oracle_params *p, const float *sigma, const float *eps_s, const float *eps_i,
                     const float *tau, float *rpx0, float *rpy0, float *rpz0,
                     float *rpx_end, float *rpy_end, float *rpz_end)
{
    const int nx = p->nx, ny = p->ny, nz = p->nz;
#define MAT(arr, x, y, z) AT(arr, x, y, z)
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int l = 0; l < 2; l++) {
                int x = l;
                RPX(rpx0, l, y, z) = rp_value(p, MAT(sigma, x, y, z), MAT(eps_s, x, y, z), MAT(eps_i, x, y, z), MAT(tau, x, y, z), 0);
                x = nx - 2 + l;
                RPX(rpx_end, l, y, z) = rp_value(p, MAT(sigma, x, y, z), MAT(eps_s, x, y, z), MAT(eps_i, x, y, z), MAT(tau, x, y, z), 0);
            }
    for (int z = 0; z < nz; z++)
        for (int x = 0; x < nx; x++)
            for (int l = 0; l < 2; l++) {
                int y = l;
                RPY(rpy0, x, l, z) = rp_value(p, MAT(sigma, x, y, z), MAT(eps_s, x, y, z), MAT(eps_i, x, y, z), MAT(tau, x, y, z), 1);
                y = ny - 2 + l;
                RPY(rpy_end, x, l, z) = rp_value(p, MAT(sigma, x, y, z), MAT(eps_s, x, y, z), MAT(eps_i, x, y, z), MAT(tau, x, y, z), 1);
            }
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++)
            for (int l = 0; l < 2; l++) {
                int z = l;
                RPZ(rpz0, x, y, l) = rp_value(p, MAT(sigma, x, y, z), MAT(eps_s, x, y, z), MAT(eps_i, x, y, z), MAT(tau, x, y, z), 1);
                z = nz - 2 + l;
                RPZ(rpz_end, x, y, l) = rp_value(p, MAT(sigma, x, y, z), MAT(eps_s, x, y, z), MAT(eps_i, x, y, z), MAT(tau, x, y, z), 1);
            }
#undef MAT
    return 0;
}

/* loadMaterials (fdtd.cu:875-939).  oracle_read_specs is its mat_specs part
 * (:880-904): at most 94 records are read; a record that fails to scan
 * re-stores the previous one; reading stops after a code >= 94.  specs
 * receives 256 x 4 floats (sigma, eps_s, eps_i, tau).
 * oracle_load_materials then reads nz slices <dir>/v1_%05d.pgm (1-based) are read: a 6-token header, then
 * nx*ny codes as one flat stream, x fastest.  codes may be NULL. */
int oracle_read_specs(const char *specs_path, float *specs)
{
    char tmp[1024];
    memset(specs, 0, sizeof(float) * 4 * ORACLE_SPEC_CODES);
    FILE *f = fopen(specs_path, "r");
    if (!f)
        return -1;
    int index = -1;
    float sv = 0, esv = 0, eiv = 0, tv = 0;
    for (int i = 0; i < 94; i++) {
        (void)fscanf(f, "%d %1023s %g %g %g %g\n", &index, tmp, &sv, &esv, &eiv, &tv);
        if (index < 0 || index >= ORACLE_SPEC_CODES) {
            fclose(f);
            return -2;
        }
        specs[index * 4 + 0] = sv;
        specs[index * 4 + 1] = esv;
        specs[index * 4 + 2] = eiv;
        specs[index * 4 + 3] = tv;
        if (index >= 94)
            break;
    }
    fclose(f);
    return 0;
}

int oracle_load_materials(const oracle_params *p, const char *specs_path, const char *dir,
                          float *specs, uint8_t *codes, float *sigma, float *eps_s, float *eps_i, float *tau)
{
    char tmp[1024];
    const int rs = oracle_read_specs(specs_path, specs);
    if (rs != 0)
        return rs;
    const size_t plane = (size_t)p->nx * p->ny;
    for (int z = 0; z < p->nz; z++) {
        char name[2100];
        snprintf(name, sizeof name, "%s/v1_%05d.pgm", dir, z + 1);
        FILE *g = fopen(name, "r");
        if (!g)
            return -3;
        int w, h;
        if (fscanf(g, "%1023s %1023s %1023s %d %d %1023s", tmp, tmp, tmp, &w, &h, tmp) != 6) {
            fclose(g);
            return -4;
        }
        for (size_t k = 0; k < plane; k++) {
            int code;
            if (fscanf(g, "%d", &code) != 1 || code < 0 || code >= ORACLE_SPEC_CODES) {
                fclose(g);
                return -5;
            }
            const size_t i = (size_t)z * plane + k;
            if (codes)
                codes[i] = (uint8_t)code;
            sigma[i] = specs[code * 4 + 0];
            eps_s[i] = specs[code * 4 + 1];
            eps_i[i] = specs[code * 4 + 2];
            tau[i] = specs[code * 4 + 3];
        }
        fclose(g);
    }
    return 0;
}

/* writeResults3d (fdtd.cu:1288-1494): for H, D, E and x, y, z, one text file
 * per z plane named <out>/{H|D|E}_field_{x|y|z}_%05d_z%05d.out holding ny
 * lines of nx values " % 9.3E". */
int oracle_write_snapshot3d(const char *out_dir, int nx, int ny, int nz, const float *const fields[9], int iteration)
{
    static const char groups[3] = {'H', 'D', 'E'};
    static const char comps[3] = {'x', 'y', 'z'};
    char name[2200];
    for (int g = 0; g < 3; g++)
        for (int c = 0; c < 3; c++) {
            const float *v = fields[g * 3 + c];
            for (int z = 0; z < nz; z++) {
                snprintf(name, sizeof name, "%s/%c_field_%c_%05d_z%05d.out", out_dir, groups[g], comps[c], iteration, z);
                FILE *f = fopen(name, "w");
                if (!f)
                    return -1;
                for (int y = 0; y < ny; y++) {
                    for (int x = 0; x < nx; x++)
                        fprintf(f, " % 9.3E", AT(v, x, y, z));
                    fprintf(f, "\n");
                }
                fclose(f);
            }
        }
    return 0;
}
