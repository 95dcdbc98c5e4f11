/*
 * ref_host.cu -- C entry points over the reference's own host set-up code.
 *
 * Test infrastructure only.  Linked with the reference's fdtd.cu (compiled
 * with ref_shim_host.h force-included and its main renamed), utils.cu and
 * fdtd_calculations.cu.  These wrappers call initParamsWithPath, setupSources,
 * loadMaterials and writeResults3d unchanged, so golden fixtures for the
 * parsers, the source table, voxelisation and the snapshot layout come from
 * the reference itself.
 *
 * loadMaterials writes specs[code*4..+3] before checking code >= 94
 * (fdtd.cu:897-903): with a code-94 record that write lands past its 94x4
 * heap buffer.  Callers of ref_host_load_materials therefore pass specs files
 * whose codes are all below 94.
 */
#include <cstring>
#include <cstdlib>
#include "fdtd.h"

/* Same layout as oracle_params in fdtd_oracle.c. */
struct ref_flat_params {
    int nx, ny, nz;
    int iterations;
    char input_path[1024];
    char output_path[1024];
    int elements_per_wave;
    float wave_frequency, pulse_width, pulse_modulation_frequency;
    int nsources;
    int sources[3 * 64];
    float default_sigma, default_eps_s, default_eps_i, default_tau_d;
    float pi, c, timeskip, lambda, dt, dx, dy, dz, mu0, eps0;
};

static void to_fdtd(const ref_flat_params *f, FdtdParams *p)
{
    memset(p, 0, sizeof *p);
    p->nx = f->nx; p->ny = f->ny; p->nz = f->nz;
    p->iterationsCount = f->iterations;
    p->inputPath = const_cast<char *>(f->input_path);
    p->outputPath = const_cast<char *>(f->output_path);
    p->elementsPerWave = f->elements_per_wave;
    p->waveFrequency = f->wave_frequency;
    p->pulseWidth = f->pulse_width;
    p->pulseModulationFrequency = f->pulse_modulation_frequency;
    p->sourcesCount = f->nsources;
    p->sources = const_cast<int *>(f->sources);
    p->defaultSigma = f->default_sigma; p->defaultEpsS = f->default_eps_s;
    p->defaultEpsI = f->default_eps_i; p->defaultTauD = f->default_tau_d;
    p->pi = f->pi; p->c = f->c; p->timeskip = f->timeskip; p->lambda = f->lambda;
    p->dt = f->dt; p->dx = f->dx; p->dy = f->dy; p->dz = f->dz;
    p->mu0 = f->mu0; p->eps0 = f->eps0;
}

extern "C" {

int ref_host_params_read(const char *path, ref_flat_params *out)
{
    FdtdParams *p = initParamsWithPath(path);
    memset(out, 0, sizeof *out);
    if (p->sourcesCount > 64) return -1;
    out->nx = p->nx; out->ny = p->ny; out->nz = p->nz;
    out->iterations = p->iterationsCount;
    strncpy(out->input_path, p->inputPath, 1023);
    strncpy(out->output_path, p->outputPath, 1023);
    out->elements_per_wave = p->elementsPerWave;
    out->wave_frequency = p->waveFrequency;
    out->pulse_width = p->pulseWidth;
    out->pulse_modulation_frequency = p->pulseModulationFrequency;
    out->nsources = p->sourcesCount;
    memcpy(out->sources, p->sources, sizeof(int) * 3 * p->sourcesCount);
    out->default_sigma = p->defaultSigma; out->default_eps_s = p->defaultEpsS;
    out->default_eps_i = p->defaultEpsI; out->default_tau_d = p->defaultTauD;
    out->pi = p->pi; out->c = p->c; out->timeskip = p->timeskip; out->lambda = p->lambda;
    out->dt = p->dt; out->dx = p->dx; out->dy = p->dy; out->dz = p->dz;
    out->mu0 = p->mu0; out->eps0 = p->eps0;
    free(p->sources);
    deallocParams(p);
    return 0;
}

int ref_host_setup_sources(const ref_flat_params *f, float *jz_out)
{
    FdtdParams p;
    to_fdtd(f, &p);
    setupSources(&p);
    memcpy(jz_out, p.jz, sizeof(float) * p.jzCount);
    free(p.jz);
    return p.jzCount;
}

int ref_host_load_materials(const ref_flat_params *f, const char *specs, const char *dir,
                            float *sigma, float *eps_s, float *eps_i, float *tau)
{
    FdtdParams p;
    to_fdtd(f, &p);
    FdtdField field;
    memset(&field, 0, sizeof field);
    field.sigma = sigma; field.epsS = eps_s; field.epsI = eps_i; field.tauD = tau;
    loadMaterials(&p, &field, specs, dir);
    return 0;
}

/* writeResults3d frees its nine buffers when done (fdtd.cu:1482-1493), so it
 * receives malloc'd copies. */
int ref_host_write_snapshot3d(const ref_flat_params *f, float **fields, int iteration)
{
    FdtdParams p;
    to_fdtd(f, &p);
    const size_t n = (size_t)f->nx * f->ny * f->nz;
    float *c[9];
    for (int k = 0; k < 9; k++) {
        c[k] = (float *)malloc(sizeof(float) * n);
        memcpy(c[k], fields[k], sizeof(float) * n);
    }
    writeResults3d(&p, c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], c[8], iteration);
    return 0;
}

}  // extern "C"
