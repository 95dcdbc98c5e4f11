// host_io.cpp -- the reference's input formats and snapshot layout on the host.
//
// Each function replaces one host routine of rafalgrodzinski/fdtd and keeps
// its observable behaviour (same scanning rules, same float/double mix in the
// derived constants, same bytes in the output files); file:line citations are
// given per function.  Parsing and formatting run on a pool of host threads.
#include "fdtd_internal.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include <sys/stat.h>
#include <thread>
#include <vector>

namespace fdtd {

int host_threads(int requested)
{
    if (requested > 0)
        return requested;
    unsigned n = std::thread::hardware_concurrency();
    return n ? static_cast<int>(n) : 4;
}

void parallel_for(int n, int nthreads, const std::function<void(int)> &fn)
{
    nthreads = std::max(1, std::min(host_threads(nthreads), n));
    if (nthreads == 1) {
        for (int i = 0; i < n; i++)
            fn(i);
        return;
    }
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    pool.reserve(nthreads);
    for (int t = 0; t < nthreads; t++)
        pool.emplace_back([&] {
            for (int i = next++; i < n; i = next++)
                fn(i);
        });
    for (auto &th : pool)
        th.join();
}

// Derived constants of initParamsWithPath (fdtd.cu:625-634); every value is
// computed in double (or float where the reference multiplies float members)
// and stored into a float member.
static void derive_constants(FdtdParams *p, float timeskip)
{
    p->pi = std::acos(-1.0);
    p->c = 3.0 * std::pow(10.0, 8.0);
    p->timeskip = timeskip;
    p->lambda = p->c / p->waveFrequency;
    p->dx = p->lambda / p->elementsPerWave;
    p->dy = p->dx;
    p->dz = p->dx;
    p->dt = 1.0 * p->timeskip /
            (p->c * std::sqrt(1.0 / std::pow((double)p->dx, 2.0) + 1.0 / std::pow((double)p->dy, 2.0) +
                              1.0 / std::pow((double)p->dz, 2.0)));
    p->mu0 = 4.0 * p->pi * std::pow(10.0, -7.0);
    p->eps0 = 1.0 / (p->mu0 * p->c * p->c);  // float product, as in the reference
}

}  // namespace fdtd

using namespace fdtd;

extern "C" {

const char *fdtd_status_string(int status)
{
    switch (status) {
    case FDTD_OK: return "success";
    case FDTD_ERR_INVALID: return "invalid argument or size";
    case FDTD_ERR_IO: return "file could not be opened, read or written";
    case FDTD_ERR_FORMAT: return "input file does not follow the reference format";
    case FDTD_ERR_NO_SYMBOLS: return "fdtd_copy_symbols has not been called on this device";
    case FDTD_ERR_NOMEM: return "host allocation failed";
    case FDTD_ERR_STATE: return "call not valid in the current state";
    case FDTD_ERR_DEVICE_TIMEOUT: return "a kernel gave up a bounded wait; results are invalid";
    case FDTD_ERR_BUSY: return "the queued work has not finished yet";
    default: return cuda_error_string(status);
    }
}

// initParamsWithPath (fdtd.cu:547-637): the lines are read in a fixed order
// with the reference's scanf formats; keys are read and discarded.
int fdtd_params_read(const char *path, FdtdParams *out)
{
    if (!path || !out)
        return FDTD_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    FILE *f = std::fopen(path, "r");
    if (!f)
        return FDTD_ERR_IO;
    char tmp[1024];
    char in_path[1024] = {0}, out_path[1024] = {0};
    FdtdParams p;
    std::memset(&p, 0, sizeof p);
    bool ok = true;
    auto skip_line = [&] { ok = ok && std::fgets(tmp, sizeof tmp, f) != nullptr; };
    ok = ok && std::fscanf(f, "%1023s %d %d %d\n", tmp, &p.nx, &p.ny, &p.nz) == 4;
    ok = ok && std::fscanf(f, "%1023s %d\n", tmp, &p.iterationsCount) == 2;
    skip_line();                                                        // nf
    ok = ok && std::fscanf(f, "%1023s %1023s\n", tmp, in_path) == 2;     // env_set_dir
    skip_line();                                                        // env_file_prefix
    ok = ok && std::fscanf(f, "%1023s %1023s\n", tmp, out_path) == 2;    // output_dir
    for (int k = 0; k < 9; k++)                                         // output_format .. source_type
        skip_line();
    ok = ok && std::fscanf(f, "%1023s %d\n", tmp, &p.elementsPerWave) == 2;
    ok = ok && std::fscanf(f, "%1023s %g\n", tmp, &p.waveFrequency) == 2;
    ok = ok && std::fscanf(f, "%1023s %g\n", tmp, &p.pulseWidth) == 2;
    ok = ok && std::fscanf(f, "%1023s %g\n", tmp, &p.pulseModulationFrequency) == 2;
    ok = ok && std::fscanf(f, "%1023s %d\n", tmp, &p.sourcesCount) == 2;
    if (!ok || p.sourcesCount < 0 || p.sourcesCount > 4096) {
        std::fclose(f);
        return FDTD_ERR_FORMAT;
    }
    std::vector<int> src(3 * (size_t)p.sourcesCount);
    for (int k = 0; k < p.sourcesCount; k++) {
        ok = ok && std::fscanf(f, "%1023s %d %d %d\n", tmp, &src[3 * k], &src[3 * k + 1], &src[3 * k + 2]) == 4;
        for (int c = 0; c < 3; c++)
            src[3 * k + c] -= 1;  // 1-based in the file (fdtd.cu:607-609)
    }
    skip_line();  // pulse_type
    ok = ok && std::fscanf(f, "%1023s %f\n", tmp, &p.defaultSigma) == 2;
    ok = ok && std::fscanf(f, "%1023s %f\n", tmp, &p.defaultEpsS) == 2;
    ok = ok && std::fscanf(f, "%1023s %f\n", tmp, &p.defaultEpsI) == 2;
    ok = ok && std::fscanf(f, "%1023s %f\n", tmp, &p.defaultTauD) == 2;
    std::fclose(f);
    if (!ok || p.nx <= 0 || p.ny <= 0 || p.nz <= 0 || p.elementsPerWave <= 0)
        return FDTD_ERR_FORMAT;
    p.iterationsCount = ((p.iterationsCount - 1) / 3 + 1) * 3;  // multiple of 3 (fdtd.cu:563)
    derive_constants(&p, 1.0f);
    p.inputPath = strdup(in_path);
    p.outputPath = strdup(out_path);
    p.sources = static_cast<int *>(std::malloc(sizeof(int) * std::max<size_t>(1, src.size())));
    if (!p.inputPath || !p.outputPath || !p.sources) {
        fdtd_params_free(&p);
        return FDTD_ERR_NOMEM;
    }
    if (!src.empty())
        std::memcpy(p.sources, src.data(), sizeof(int) * src.size());
    *out = p;
    return FDTD_OK;
}

int fdtd_params_set_timeskip(FdtdParams *p, float timeskip)
{
    if (!p || !(timeskip > 0.0f) || p->elementsPerWave <= 0 || !(p->waveFrequency > 0.0f))
        return FDTD_ERR_INVALID;
    derive_constants(p, timeskip);
    return FDTD_OK;
}

void fdtd_params_free(FdtdParams *p)
{
    if (!p)
        return;
    std::free(p->inputPath);
    std::free(p->outputPath);
    std::free(p->sources);
    std::free(p->jz);
    p->inputPath = p->outputPath = nullptr;
    p->sources = nullptr;
    p->jz = nullptr;
    p->jzCount = 0;
}

// setupSources (fdtd.cu:1027-1082).  Sample spacing `fine` and half-width
// `half` are truncated like the reference's int assignments; the Gaussian is
// sampled every `fine` fine steps from the first sample with |g| >= 1e-9,
// scaled by 1e-15/dt/3, then differenced over two samples and divided by
// dx*dy.  Entries past the first 2^14 keep the undifferenced samples, as in
// the reference (its second pass stops at 1 << 14).
int fdtd_setup_sources(FdtdParams *p)
{
    if (!p || !(p->dt > 0.0f))
        return FDTD_ERR_INVALID;
    const int off = FDTD_JZ_LEN;
    std::vector<float> g((size_t)off * 2, 0.0f), g2((size_t)off * 2, 0.0f);
    float *jz = static_cast<float *>(std::calloc(off, sizeof(float)));
    if (!jz)
        return FDTD_ERR_NOMEM;
    const int fine = (1 << 13) * p->pulseWidth * p->waveFrequency * p->dt;
    const int half = 1.0 / (p->pulseWidth * p->waveFrequency) / (p->dt / fine) / 2.0;
    if (fine <= 0 || half < 0 || half + 2 >= off) {
        std::free(jz);
        return FDTD_ERR_INVALID;
    }
    for (int i = -half - 1; i <= half + 1; i++) {
        const float v1 = ((float)i / (((float)half + 1.0) / 4.0));
        const float v2 = std::exp(-std::pow((double)v1, 2.0));
        const float v3 = std::cos(2.0 * std::acos(-1.0) * p->pulseModulationFrequency * p->waveFrequency * i *
                                  (double)(p->dt / fine));
        g[i + off] = v2 * v3;
    }
    int start = 0;
    bool found = false;
    for (int i = -(1 << 12); i < (1 << 12); i++)
        if (std::fabs(g[i + off]) >= 1e-9 && i % fine == 0) {
            start = i;
            found = true;
            break;
        }
    if (!found) {
        std::free(jz);
        return FDTD_ERR_INVALID;
    }
    int n = 0;
    for (int i = start; i <= half + 1 && n < off; i += fine)
        jz[n++] = g[i + off] * 1e-15 / p->dt / 3.0;
    for (int i = 2; i <= (1 << 14); i++) {
        const float d1 = (jz[i] - jz[i - 1]) / p->dt;
        const float d0 = (jz[i - 1] - jz[i - 2]) / p->dt;
        g2[i - 1 + off] = (d1 + d0) / 2.0 * (p->dt * p->dz) / (p->dx * p->dy * p->dz);
    }
    for (int i = 0; i < (1 << 14); i++)
        jz[i] = g2[i + off + 1];
    std::free(p->jz);
    p->jz = jz;
    p->jzCount = off;
    return FDTD_OK;
}

}  // extern "C"

namespace fdtd {

// One Mur slab value (fdtd.cu:959-963 and mirrors): Re(eps_i +
// (eps_s - eps_i)/(1 + c1) - c2) where c1, c2 are C99 `float complex`
// values -- real for the x slabs, times i for the y and z slabs -- and the
// rest is evaluated in double complex.  std::complex<double> uses the same
// complex division routine as C99 complex arithmetic.
float mur_rp_value(const FdtdParams *p, float sigma, float eps_s, float eps_i, float tau, bool imaginary)
{
    const double w = 2.0 * p->pi * p->waveFrequency * tau;
    const double s = sigma / (2.0 * p->pi * p->waveFrequency * p->eps0);
    const std::complex<float> c1 = imaginary ? std::complex<float>(0.0f, (float)w) : std::complex<float>((float)w, 0.0f);
    const std::complex<float> c2 = imaginary ? std::complex<float>(0.0f, (float)s) : std::complex<float>((float)s, 0.0f);
    const std::complex<double> den(1.0 + (double)c1.real(), (double)c1.imag());
    const std::complex<double> q = (double)(eps_s - eps_i) / den;
    const std::complex<double> r = ((double)eps_i + q) - std::complex<double>(c2.real(), c2.imag());
    return (float)r.real();
}

}  // namespace fdtd

extern "C" {

// setupMurBoundary (fdtd.cu:942-1024).
int fdtd_setup_mur(const FdtdParams *p, const float *sigma, const float *epsS, const float *epsI, const float *tauD,
                   float *rpx0, float *rpy0, float *rpz0, float *rpxEnd, float *rpyEnd, float *rpzEnd)
{
    if (!p || !sigma || !epsS || !epsI || !tauD || !rpx0 || !rpy0 || !rpz0 || !rpxEnd || !rpyEnd || !rpzEnd)
        return FDTD_ERR_INVALID;
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    if (nx < 2 || ny < 2 || nz < 2)
        return FDTD_ERR_INVALID;
    auto cell = [&](int x, int y, int z) { return ((size_t)z * ny + y) * nx + x; };
    auto val = [&](size_t i, bool imag) { return mur_rp_value(p, sigma[i], epsS[i], epsI[i], tauD[i], imag); };
    parallel_for(nz, 0, [&](int z) {
        for (int y = 0; y < ny; y++)
            for (int l = 0; l < 2; l++) {
                rpx0[((size_t)z * ny + y) * 2 + l] = val(cell(l, y, z), false);
                rpxEnd[((size_t)z * ny + y) * 2 + l] = val(cell(nx - 2 + l, y, z), false);
            }
        for (int x = 0; x < nx; x++)
            for (int l = 0; l < 2; l++) {
                rpy0[((size_t)z * 2 + l) * nx + x] = val(cell(x, l, z), true);
                rpyEnd[((size_t)z * 2 + l) * nx + x] = val(cell(x, ny - 2 + l, z), true);
            }
    });
    for (int l = 0; l < 2; l++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                rpz0[((size_t)l * ny + y) * nx + x] = val(cell(x, y, l), true);
                rpzEnd[((size_t)l * ny + y) * nx + x] = val(cell(x, y, nz - 2 + l), true);
            }
    return FDTD_OK;
}

int fdtd_setup_mur_uniform(const FdtdParams *p, float sigma, float epsS, float epsI, float tauD, float *rpx0,
                           float *rpy0, float *rpz0, float *rpxEnd, float *rpyEnd, float *rpzEnd)
{
    if (!p || !rpx0 || !rpy0 || !rpz0 || !rpxEnd || !rpyEnd || !rpzEnd || p->nx < 2 || p->ny < 2 || p->nz < 2)
        return FDTD_ERR_INVALID;
    const float vx = mur_rp_value(p, sigma, epsS, epsI, tauD, false);
    const float vyz = mur_rp_value(p, sigma, epsS, epsI, tauD, true);
    const size_t sx = 2 * (size_t)p->ny * p->nz, sy = (size_t)p->nx * 2 * p->nz, sz = (size_t)p->nx * p->ny * 2;
    std::fill(rpx0, rpx0 + sx, vx);
    std::fill(rpxEnd, rpxEnd + sx, vx);
    std::fill(rpy0, rpy0 + sy, vyz);
    std::fill(rpyEnd, rpyEnd + sy, vyz);
    std::fill(rpz0, rpz0 + sz, vyz);
    std::fill(rpzEnd, rpzEnd + sz, vyz);
    return FDTD_OK;
}

// The mat_specs half of loadMaterials (fdtd.cu:878-904).  fscanf keeps the
// reference's partial-assignment behaviour on a line that does not scan.
int fdtd_read_specs(const char *specsPath, float *specs)
{
    if (!specsPath || !specs)
        return FDTD_ERR_INVALID;
    std::memset(specs, 0, sizeof(float) * 4 * FDTD_MAX_CLASSES);
    FILE *f = std::fopen(specsPath, "r");
    if (!f)
        return FDTD_ERR_IO;
    char tmp[1024];
    int index = -1;
    float sv = 0, esv = 0, eiv = 0, tv = 0;
    for (int i = 0; i < 94; i++) {
        (void)std::fscanf(f, "%d %1023s %g %g %g %g\n", &index, tmp, &sv, &esv, &eiv, &tv);
        if (index < 0 || index >= FDTD_MAX_CLASSES) {
            std::fclose(f);
            return FDTD_ERR_FORMAT;
        }
        specs[index * 4 + 0] = sv;
        specs[index * 4 + 1] = esv;
        specs[index * 4 + 2] = eiv;
        specs[index * 4 + 3] = tv;
        if (index >= 94)
            break;
    }
    std::fclose(f);
    return FDTD_OK;
}

}  // extern "C"

namespace fdtd {

// Reads one PGM slice the way loadMaterials does (fdtd.cu:911-935): six
// header tokens ("%s %s %s %d %d %s"), then nx*ny decimal codes as a flat
// stream.  The whole file is read at once and parsed without scanf.
static int read_slice(const std::string &name, size_t count, uint8_t *dst)
{
    FILE *f = std::fopen(name.c_str(), "rb");
    if (!f)
        return FDTD_ERR_IO;
    std::fseek(f, 0, SEEK_END);
    long len = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (len < 0) {
        std::fclose(f);
        return FDTD_ERR_IO;
    }
    std::string buf((size_t)len, '\0');
    size_t got = len ? std::fread(&buf[0], 1, (size_t)len, f) : 0;
    std::fclose(f);
    if (got != (size_t)len)
        return FDTD_ERR_IO;
    const char *s = buf.data(), *end = s + buf.size();
    auto is_space = [](char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; };
    auto skip_ws = [&] { while (s < end && is_space(*s)) s++; };
    auto parse_int = [&](long *v) -> bool {
        skip_ws();
        bool neg = false;
        if (s < end && (*s == '+' || *s == '-')) {
            neg = *s == '-';
            s++;
        }
        if (s >= end || *s < '0' || *s > '9')
            return false;
        long acc = 0;
        while (s < end && *s >= '0' && *s <= '9') {
            if (acc < 100000000L)
                acc = acc * 10 + (*s - '0');
            s++;
        }
        *v = neg ? -acc : acc;
        return true;
    };
    auto skip_token = [&]() -> bool {
        skip_ws();
        if (s >= end)
            return false;
        while (s < end && !is_space(*s))
            s++;
        return true;
    };
    long w, h;
    if (!skip_token() || !skip_token() || !skip_token() || !parse_int(&w) || !parse_int(&h) || !skip_token())
        return FDTD_ERR_FORMAT;
    for (size_t k = 0; k < count; k++) {
        long v;
        if (!parse_int(&v) || v < 0 || v >= FDTD_MAX_CLASSES)
            return FDTD_ERR_FORMAT;
        dst[k] = (uint8_t)v;
    }
    return FDTD_OK;
}

}  // namespace fdtd

extern "C" {

int fdtd_load_material_codes(const FdtdParams *p, const char *materialsPath, uint8_t *codes, int nthreads)
{
    if (!p || !materialsPath || !codes || p->nx <= 0 || p->ny <= 0 || p->nz <= 0)
        return FDTD_ERR_INVALID;
    const size_t plane = (size_t)p->nx * p->ny;
    std::vector<int> status(p->nz, FDTD_OK);
    parallel_for(p->nz, nthreads, [&](int z) {
        char name[64];
        std::snprintf(name, sizeof name, "/v1_%05d.pgm", z + 1);
        status[z] = read_slice(std::string(materialsPath) + name, plane, codes + (size_t)z * plane);
    });
    for (int st : status)
        if (st != FDTD_OK)
            return st;
    return FDTD_OK;
}

int fdtd_load_material_codes_cached(const FdtdParams *p, const char *materialsPath, const char *cachePath,
                                    uint8_t *codes, int nthreads, int *fromCache)
{
    if (fromCache)
        *fromCache = 0;
    if (!p || !materialsPath || !cachePath || !codes || p->nx <= 0 || p->ny <= 0 || p->nz <= 0)
        return FDTD_ERR_INVALID;
    // fingerprint of the slice files: FNV-1a over the dimensions and each
    // slice's size and modification time (a missing slice makes the parse fail)
    unsigned long long fp = 1469598103934665603ULL;
    auto mix = [&](unsigned long long v) {
        for (int b = 0; b < 8; b++)
            fp = (fp ^ ((v >> (8 * b)) & 0xffu)) * 1099511628211ULL;
    };
    mix((unsigned long long)p->nx);
    mix((unsigned long long)p->ny);
    mix((unsigned long long)p->nz);
    for (int z = 0; z < p->nz; z++) {
        char name[64];
        std::snprintf(name, sizeof name, "/v1_%05d.pgm", z + 1);
        struct stat sb;
        if (stat((std::string(materialsPath) + name).c_str(), &sb) != 0)
            return FDTD_ERR_IO;
        mix((unsigned long long)sb.st_size);
        mix((unsigned long long)sb.st_mtim.tv_sec);
        mix((unsigned long long)sb.st_mtim.tv_nsec);
    }
    static const char MAGIC[8] = {'F', 'D', 'T', 'D', 'U', '8', 'V', '1'};
    struct Header {
        char magic[8];
        int32_t nx, ny, nz, pad;
        uint64_t fingerprint;
    };
    const size_t n = (size_t)p->nx * p->ny * p->nz;
    if (FILE *f = std::fopen(cachePath, "rb")) {
        Header h{};
        const bool hit = std::fread(&h, sizeof h, 1, f) == 1 && std::memcmp(h.magic, MAGIC, 8) == 0 &&
                         h.nx == p->nx && h.ny == p->ny && h.nz == p->nz && h.fingerprint == fp &&
                         std::fread(codes, 1, n, f) == n;
        std::fclose(f);
        if (hit) {
            if (fromCache)
                *fromCache = 1;
            return FDTD_OK;
        }
    }
    const int st = fdtd_load_material_codes(p, materialsPath, codes, nthreads);
    if (st != FDTD_OK)
        return st;
    // write beside the target and rename, so a reader never sees half a cache
    const std::string tmp = std::string(cachePath) + ".tmp";
    if (FILE *f = std::fopen(tmp.c_str(), "wb")) {
        Header h{};
        std::memcpy(h.magic, MAGIC, 8);
        h.nx = p->nx;
        h.ny = p->ny;
        h.nz = p->nz;
        h.fingerprint = fp;
        const bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 && std::fwrite(codes, 1, n, f) == n;
        if (std::fclose(f) == 0 && ok)
            std::rename(tmp.c_str(), cachePath);
        else
            std::remove(tmp.c_str());
    }
    return FDTD_OK;
}

int fdtd_load_materials(const FdtdParams *p, const char *specsPath, const char *materialsPath, float *sigma,
                        float *epsS, float *epsI, float *tauD)
{
    if (!p || !sigma || !epsS || !epsI || !tauD)
        return FDTD_ERR_INVALID;
    std::vector<float> specs(4 * FDTD_MAX_CLASSES);
    int st = fdtd_read_specs(specsPath, specs.data());
    if (st != FDTD_OK)
        return st;
    const size_t n = (size_t)p->nx * p->ny * p->nz;
    std::vector<uint8_t> codes(n);
    st = fdtd_load_material_codes(p, materialsPath, codes.data(), 0);
    if (st != FDTD_OK)
        return st;
    for (size_t i = 0; i < n; i++) {
        const float *s = &specs[codes[i] * 4];
        sigma[i] = s[0];
        epsS[i] = s[1];
        epsI[i] = s[2];
        tauD[i] = s[3];
    }
    return FDTD_OK;
}

}  // extern "C"

namespace fdtd {

// Appends " " followed by printf("% 9.3E", v) for a float v.  Finite values
// whose 4-digit rounding is not near a tie are formatted directly; anything
// else (ties, subnormals, infinities, NaNs) goes through snprintf, so the
// bytes always equal the reference's fprintf output (fdtd.cu:1313).
static inline void append_value(std::string &out, float fv)
{
    const double v = fv;
    const double a = std::fabs(v);
    if (std::isfinite(v) && a >= 1e-37) {
        int e = (int)std::floor(std::log10(a));
        double scaled = a * std::pow(10.0, 3 - e);  // ~[1000, 10000)
        if (scaled < 1000.0) {
            scaled *= 10.0;
            e -= 1;
        } else if (scaled >= 10000.0) {
            scaled /= 10.0;
            e += 1;
        }
        const double fl = std::floor(scaled);
        const double frac = scaled - fl;
        if (std::fabs(frac - 0.5) > 1e-6 && scaled > 1000.0 + 1e-6 && scaled < 9999.5 - 1e-6) {
            long m = (long)fl + (frac > 0.5 ? 1 : 0);
            if (m >= 10000) {
                m /= 10;
                e += 1;
            }
            if (m >= 1000 && m < 10000 && e >= -99 && e <= 99) {
                char b[16];
                int k = 0;
                b[k++] = ' ';
                b[k++] = std::signbit(v) ? '-' : ' ';
                b[k++] = (char)('0' + m / 1000);
                b[k++] = '.';
                b[k++] = (char)('0' + (m / 100) % 10);
                b[k++] = (char)('0' + (m / 10) % 10);
                b[k++] = (char)('0' + m % 10);
                b[k++] = 'E';
                b[k++] = e < 0 ? '-' : '+';
                const int ae = e < 0 ? -e : e;
                b[k++] = (char)('0' + ae / 10);
                b[k++] = (char)('0' + ae % 10);
                out.append(b, k);
                return;
            }
        }
    }
    char b[64];
    const int k = std::snprintf(b, sizeof b, " % 9.3E", v);
    out.append(b, (size_t)k);
}

int write_plane_text(const std::string &path, const float *plane, int nx, int ny)
{
    std::string out;
    out.reserve((size_t)nx * ny * 11 + ny);
    for (int y = 0; y < ny; y++) {
        const float *row = plane + (size_t)y * nx;
        for (int x = 0; x < nx; x++)
            append_value(out, row[x]);
        out.push_back('\n');
    }
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f)
        return FDTD_ERR_IO;
    const size_t w = std::fwrite(out.data(), 1, out.size(), f);
    const int rc = std::fclose(f);
    return (w == out.size() && rc == 0) ? FDTD_OK : FDTD_ERR_IO;
}

std::string snapshot_name_f32(const char *dir, int field, int iteration, int z0, int nplanes)
{
    static const char groups[3] = {'H', 'D', 'E'};
    static const char comps[3] = {'x', 'y', 'z'};
    char name[112];
    std::snprintf(name, sizeof name, "/%c_field_%c_%05d_z%05d_n%05d.f32", groups[field / 3], comps[field % 3],
                  iteration, z0, nplanes);
    return std::string(dir) + name;
}

int write_floats(const std::string &path, const float *data, size_t count)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f)
        return FDTD_ERR_IO;
    // the hosts this builds for (x86-64, aarch64) are little-endian: the bytes
    // in memory are the file's bytes
    const bool ok = std::fwrite(data, sizeof(float), count, f) == count;
    return std::fclose(f) == 0 && ok ? FDTD_OK : FDTD_ERR_IO;
}

std::string snapshot_name(const char *dir, int field, int iteration, int z)
{
    static const char groups[3] = {'H', 'D', 'E'};
    static const char comps[3] = {'x', 'y', 'z'};
    char name[96];
    std::snprintf(name, sizeof name, "/%c_field_%c_%05d_z%05d.out", groups[field / 3], comps[field % 3], iteration, z);
    return std::string(dir) + name;
}

}  // namespace fdtd

extern "C" {

// writeResults3d (fdtd.cu:1288-1494): files in the reference's order.
int fdtd_write_results3d(const FdtdParams *p, const float *hx, const float *hy, const float *hz, const float *dx,
                         const float *dy, const float *dz, const float *ex, const float *ey, const float *ez,
                         int iteration, int nthreads)
{
    if (!p || !p->outputPath || p->nx <= 0 || p->ny <= 0 || p->nz <= 0)
        return FDTD_ERR_INVALID;
    const float *fields[9] = {hx, hy, hz, dx, dy, dz, ex, ey, ez};
    const size_t plane = (size_t)p->nx * p->ny;
    std::vector<int> jobs;
    for (int f = 0; f < 9; f++)
        if (fields[f])
            for (int z = 0; z < p->nz; z++)
                jobs.push_back(f * p->nz + z);
    std::vector<int> status(jobs.size(), FDTD_OK);
    parallel_for((int)jobs.size(), nthreads, [&](int j) {
        const int f = jobs[j] / p->nz, z = jobs[j] % p->nz;
        status[j] = write_plane_text(snapshot_name(p->outputPath, f, iteration, z), fields[f] + (size_t)z * plane,
                                     p->nx, p->ny);
    });
    for (int st : status)
        if (st != FDTD_OK)
            return st;
    return FDTD_OK;
}

}  // extern "C"
