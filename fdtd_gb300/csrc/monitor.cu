// monitor.cu -- on-device monitors of a solve (probe time series, a running
// DFT of E, spectral SAR) and checkpoint/resume.  None of this exists in the
// reference, which copies all nine fields to the host every step instead
// (fdtd.cu:134-136,176-178,221-223); these are the consumers of the loop that
// a long solve needs without that traffic.
//
// The monitor kernel runs after every step (it is captured into the step
// graphs).  It reads the device step counter, so one graph serves every step:
// block 0 appends the probes' E values; when the completed step count is a
// multiple of the DFT stride, every block adds E(t) exp(-i w t) stride dt to
// the FP64 accumulators of its cells.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "solver_internal.cuh"

using namespace fdtd;

namespace {

int cu(cudaError_t e) { return e == cudaSuccess ? FDTD_OK : (int)e; }

struct MonitorArgs {
    const int *counter;        // completed steps (advanced by the step's last kernel)
    const float *e[3];         // E after the step
    // probes
    int nprobes, probe_cap, probe_start;
    const long long *probe_idx;  // cell index of each probe (grids may exceed 2^31 cells)
    float *probe_buf;
    // DFT
    int dft_on, stride;
    double omega, wdt;         // 2 pi f, stride * dt
    double dt;
    size_t base, count;        // first cell and number of cells of the DFT planes
    double *acc;               // re x,y,z then im x,y,z (count each)
};

__global__ void __launch_bounds__(256) monitor_kernel(MonitorArgs a)
{
    const int m = *a.counter;
    if (blockIdx.x == 0 && (int)threadIdx.x < a.nprobes) {
        const int k = m - a.probe_start - 1;
        if (k >= 0 && k < a.probe_cap) {
            const int p = threadIdx.x;
            const long long idx = a.probe_idx[p];
            float *dst = a.probe_buf + ((size_t)k * a.nprobes + p) * 3;
            dst[0] = a.e[0][idx];
            dst[1] = a.e[1][idx];
            dst[2] = a.e[2][idx];
        }
    }
    if (!a.dft_on || m % a.stride != 0)
        return;
    __shared__ double cs[2];
    if (threadIdx.x == 0) {
        double sn, cn;
        sincos(-a.omega * (double)m * a.dt, &sn, &cn);
        cs[0] = cn * a.wdt;
        cs[1] = sn * a.wdt;
    }
    __syncthreads();
    const double c = cs[0], s = cs[1];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.count; i += (size_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int comp = 0; comp < 3; comp++) {
            const double e = a.e[comp][a.base + i];
            a.acc[comp * a.count + i] += e * c;
            a.acc[(3 + comp) * a.count + i] += e * s;
        }
    }
}

struct SarArgs {
    const double *acc;
    size_t base, count;
    const uint8_t *mat;
    float sigma[FDTD_MAX_CLASSES];
    float inv_2rho[FDTD_MAX_CLASSES];
    double *block_max;
    long long *block_arg;
};

__global__ void __launch_bounds__(256) sar_kernel(SarArgs a)
{
    double best = -1.0;
    long long arg = -1;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.count; i += (size_t)gridDim.x * blockDim.x) {
        double e2 = 0.0;
#pragma unroll
        for (int comp = 0; comp < 3; comp++) {
            const double re = a.acc[comp * a.count + i], im = a.acc[(3 + comp) * a.count + i];
            e2 += re * re + im * im;
        }
        const int cls = a.mat[a.base + i];
        const double sar = (double)a.sigma[cls] * e2 * (double)a.inv_2rho[cls];
        if (sar > best) {
            best = sar;
            arg = (long long)(a.base + i);
        }
    }
    __shared__ double sbest[256];
    __shared__ long long sarg[256];
    sbest[threadIdx.x] = best;
    sarg[threadIdx.x] = arg;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w && sbest[threadIdx.x + w] > sbest[threadIdx.x]) {
            sbest[threadIdx.x] = sbest[threadIdx.x + w];
            sarg[threadIdx.x] = sarg[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.block_max[blockIdx.x] = sbest[0];
        a.block_arg[blockIdx.x] = sarg[0];
    }
}

int monitor_blocks() { return 152 * 8; }

// Slot of the latest / previous E and D after `count` completed steps.
int latest_slot(int count) { return count > 0 ? ((count - 1) & 1) : 0; }
int previous_slot(int count) { return count > 0 ? (count & 1) : 1; }

}  // namespace

namespace fdtd {

int launch_monitor(fdtd_solver *s, int n)
{
    if (s->nprobes == 0 && !s->dft_on)
        return FDTD_OK;
    MonitorArgs a{};
    a.counter = s->counter;
    for (int c = 0; c < 3; c++)
        a.e[c] = s->e[n & 1][c];  // step n writes E^{n+1} into slot n % 2
    a.nprobes = s->nprobes;
    a.probe_cap = s->probe_cap;
    a.probe_start = s->probe_start;
    a.probe_idx = s->d_probe_idx;
    a.probe_buf = s->d_probe_buf;
    a.dft_on = s->dft_on ? 1 : 0;
    a.stride = s->dft_stride;
    a.omega = 2.0 * M_PI * s->dft_freq;
    a.dt = s->plan->dt;
    a.wdt = (double)s->dft_stride * s->plan->dt;
    a.base = (size_t)s->dft_z0 * s->nx * s->ny;
    a.count = (size_t)s->dft_np * s->nx * s->ny;
    a.acc = s->d_dft;
    monitor_kernel<<<s->dft_on ? monitor_blocks() : 1, 256, 0, s->stream>>>(a);
    return cu(cudaGetLastError());
}

}  // namespace fdtd

extern "C" {

int fdtd_solver_set_probes(fdtd_solver *s, int nprobes, const int *xyz, int capacity)
{
    if (!s || nprobes < 0 || nprobes > FDTD_MAX_PROBES || (nprobes > 0 && (!xyz || capacity < 1)))
        return FDTD_ERR_INVALID;
    std::vector<long long> idx(nprobes);
    for (int p = 0; p < nprobes; p++) {
        const int x = xyz[3 * p], y = xyz[3 * p + 1], z = xyz[3 * p + 2];
        if (x < 0 || x >= s->nx || y < 0 || y >= s->ny || z < 0 || z >= s->nz)
            return FDTD_ERR_INVALID;
        idx[p] = (long long)cell_index(x, y, z, s->nx, s->ny);
    }
    int st = fdtd_solver_synchronize(s);
    if (st != FDTD_OK)
        return st;
    cudaFree(s->d_probe_idx);
    cudaFree(s->d_probe_buf);
    s->d_probe_idx = nullptr;
    s->d_probe_buf = nullptr;
    s->nprobes = 0;
    reset_graphs(s);
    if (nprobes == 0)
        return FDTD_OK;
    st = cu(cudaMalloc(&s->d_probe_idx, sizeof(long long) * nprobes));
    if (st == FDTD_OK)
        st = cu(cudaMalloc(&s->d_probe_buf, sizeof(float) * 3 * (size_t)nprobes * capacity));
    if (st == FDTD_OK)
        st = cu(cudaMemcpy(s->d_probe_idx, idx.data(), sizeof(long long) * nprobes, cudaMemcpyHostToDevice));
    if (st == FDTD_OK)
        st = cu(cudaMemset(s->d_probe_buf, 0, sizeof(float) * 3 * (size_t)nprobes * capacity));
    if (st != FDTD_OK)
        return st;
    s->nprobes = nprobes;
    s->probe_cap = capacity;
    s->probe_start = s->steps;
    return FDTD_OK;
}

int fdtd_solver_get_probes(fdtd_solver *s, float *out, int *nsteps)
{
    if (!s || !nsteps)
        return FDTD_ERR_INVALID;
    int st = fdtd_solver_synchronize(s);
    if (st != FDTD_OK)
        return st;
    int k = s->steps - s->probe_start;
    if (k > s->probe_cap)
        k = s->probe_cap;
    *nsteps = s->nprobes ? k : 0;
    if (s->nprobes && k > 0 && out)
        st = cu(cudaMemcpy(out, s->d_probe_buf, sizeof(float) * 3 * (size_t)s->nprobes * k, cudaMemcpyDeviceToHost));
    return st;
}

int fdtd_solver_set_dft(fdtd_solver *s, double frequency, int stride, int z0, int nplanes)
{
    if (!s || stride < 1 || !(frequency >= 0.0))
        return FDTD_ERR_INVALID;
    if (nplanes == 0) {
        z0 = 0;
        nplanes = s->nz;
    }
    if (z0 < 0 || nplanes < 0 || z0 + nplanes > s->nz)
        return FDTD_ERR_INVALID;
    int st = fdtd_solver_synchronize(s);
    if (st != FDTD_OK)
        return st;
    cudaFree(s->d_dft);
    s->d_dft = nullptr;
    s->dft_on = false;
    reset_graphs(s);
    if (frequency == 0.0 && nplanes == 0)
        return FDTD_OK;
    const size_t count = (size_t)s->nx * s->ny * nplanes;
    st = cu(cudaMalloc(&s->d_dft, sizeof(double) * 6 * count));
    if (st == FDTD_OK)
        st = cu(cudaMemset(s->d_dft, 0, sizeof(double) * 6 * count));
    if (st != FDTD_OK)
        return st;
    s->dft_on = true;
    s->dft_freq = frequency;
    s->dft_stride = stride;
    s->dft_z0 = z0;
    s->dft_np = nplanes;
    return FDTD_OK;
}

int fdtd_solver_get_dft(fdtd_solver *s, int comp, double *re, double *im)
{
    if (!s || comp < 0 || comp > 2 || !s->dft_on)
        return FDTD_ERR_INVALID;
    int st = fdtd_solver_synchronize(s);
    const size_t count = (size_t)s->nx * s->ny * s->dft_np;
    if (st == FDTD_OK && re)
        st = cu(cudaMemcpy(re, s->d_dft + comp * count, sizeof(double) * count, cudaMemcpyDeviceToHost));
    if (st == FDTD_OK && im)
        st = cu(cudaMemcpy(im, s->d_dft + (3 + comp) * count, sizeof(double) * count, cudaMemcpyDeviceToHost));
    return st;
}

int fdtd_solver_peak_sar(fdtd_solver *s, const float *rho, double *peak, long long *cell)
{
    if (!s || !peak || !s->dft_on)
        return FDTD_ERR_INVALID;
    int st = fdtd_solver_synchronize(s);
    if (st != FDTD_OK)
        return st;
    SarArgs a{};
    a.acc = s->d_dft;
    a.base = (size_t)s->dft_z0 * s->nx * s->ny;
    a.count = (size_t)s->dft_np * s->nx * s->ny;
    a.mat = s->mat;
    for (int k = 0; k < s->nclasses; k++) {
        const float r = rho ? rho[k] : 1000.0f;
        if (!(r > 0.0f))
            return FDTD_ERR_INVALID;
        a.sigma[k] = s->specs[4 * k];
        a.inv_2rho[k] = 0.5f / r;
    }
    const int nb = monitor_blocks();
    double *bm = nullptr;
    st = cu(cudaMalloc(&bm, (sizeof(double) + sizeof(long long)) * nb));
    if (st != FDTD_OK)
        return st;
    a.block_max = bm;
    a.block_arg = reinterpret_cast<long long *>(bm + nb);
    sar_kernel<<<nb, 256, 0, s->stream>>>(a);
    std::vector<double> hm(nb);
    std::vector<long long> ha(nb);
    st = cu(cudaGetLastError());
    if (st == FDTD_OK)
        st = cu(cudaMemcpyAsync(hm.data(), a.block_max, sizeof(double) * nb, cudaMemcpyDeviceToHost, s->stream));
    if (st == FDTD_OK)
        st = cu(cudaMemcpyAsync(ha.data(), a.block_arg, sizeof(long long) * nb, cudaMemcpyDeviceToHost, s->stream));
    if (st == FDTD_OK)
        st = cu(cudaStreamSynchronize(s->stream));
    cudaFree(bm);
    if (st != FDTD_OK)
        return st;
    double best = -1.0;
    long long arg = -1;
    for (int b = 0; b < nb; b++)
        if (hm[b] > best) {
            best = hm[b];
            arg = ha[b];
        }
    *peak = best;
    if (cell)
        *cell = arg;
    return FDTD_OK;
}

// ------------------------------------------------------------- checkpoint

struct CheckpointHeader {
    char magic[8];
    uint32_t version;
    int32_t nx, ny, nz, scheme, nclasses, steps;
    uint64_t material_hash;
};

static const char CKP_MAGIC[8] = {'F', 'D', 'T', 'D', 'G', 'B', '3', 'C'};

// Checkpoint versions: 1 holds the D form's 15 arrays (either D-form
// kernel restores it), 2 the compact form's 12, 3 the 16-bit-R form's 9
// float arrays, its three FP16 residual arrays and its scale words.
static uint32_t ckp_version(const fdtd_solver *s)
{
    return s->kernel == FDTD_KERNEL_COMPACT_R16 ? 3u : s->kernel == FDTD_KERNEL_COMPACT ? 2u : 1u;
}

// The state blocks after `count` steps: H, E^n, E^{n-1}, then D^n, D^{n-1}
// (D form), R (compact form) or the FP16 residuals and the scale words.
static int state_blocks(fdtd_solver *s, int count, void *ptr[16], size_t bytes[16])
{
    const int hb = s->kernel != FDTD_KERNEL_TWO_PASS ? (count & 1) : 0;
    const int l = latest_slot(count), p = previous_slot(count);
    const size_t fb = sizeof(float) * s->ncell;
    int n = 0;
    for (int c = 0; c < 3; c++) {
        ptr[n] = s->h[hb][c];
        ptr[n + 3] = s->e[l][c];
        ptr[n + 6] = s->e[p][c];
        bytes[n] = bytes[n + 3] = bytes[n + 6] = fb;
        n++;
    }
    n = 9;
    if (s->kernel == FDTD_KERNEL_COMPACT_R16) {
        for (int c = 0; c < 3; c++, n++) {
            ptr[n] = s->d[0][c];
            bytes[n] = sizeof(uint16_t) * s->ncell;
        }
        ptr[n] = s->rexp;
        bytes[n++] = sizeof(uint32_t) * r16_words(s->nx, s->ny, s->nz);
        return n;
    }
    for (int c = 0; c < 3; c++, n++) {
        ptr[n] = s->d[l][c];
        bytes[n] = fb;
    }
    if (s->kernel != FDTD_KERNEL_COMPACT)
        for (int c = 0; c < 3; c++, n++) {
            ptr[n] = s->d[p][c];
            bytes[n] = fb;
        }
    return n;
}

int fdtd_solver_checkpoint(fdtd_solver *s, const char *path)
{
    if (!s || !path)
        return FDTD_ERR_INVALID;
    int st = fdtd_solver_synchronize(s);
    if (st != FDTD_OK)
        return st;
    FILE *f = std::fopen(path, "wb");
    if (!f)
        return FDTD_ERR_IO;
    CheckpointHeader h{};
    std::memcpy(h.magic, CKP_MAGIC, 8);
    h.version = ckp_version(s);
    h.nx = s->nx; h.ny = s->ny; h.nz = s->nz;
    h.scheme = s->scheme;
    h.nclasses = s->nclasses;
    h.steps = s->steps;
    h.material_hash = s->material_hash;
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
    void *ptr[16];
    size_t bytes[16];
    const int nb = state_blocks(s, s->steps, ptr, bytes);
    std::vector<char> buf(sizeof(float) * s->ncell);
    for (int k = 0; k < nb && ok; k++) {
        buf.resize(bytes[k]);
        st = cu(cudaMemcpy(buf.data(), ptr[k], bytes[k], cudaMemcpyDeviceToHost));
        ok = st == FDTD_OK && std::fwrite(buf.data(), 1, bytes[k], f) == bytes[k];
    }
    if (std::fclose(f) != 0)
        ok = false;
    if (st != FDTD_OK)
        return st;
    return ok ? FDTD_OK : FDTD_ERR_IO;
}

int fdtd_solver_restore(fdtd_solver *s, const char *path)
{
    if (!s || !path)
        return FDTD_ERR_INVALID;
    int st = fdtd_solver_synchronize(s);
    if (st == FDTD_OK)
        st = fdtd_solver_flush_snapshots(s);
    if (st != FDTD_OK)
        return st;
    FILE *f = std::fopen(path, "rb");
    if (!f)
        return FDTD_ERR_IO;
    CheckpointHeader h{};
    if (std::fread(&h, sizeof h, 1, f) != 1 || std::memcmp(h.magic, CKP_MAGIC, 8) != 0 || h.version != ckp_version(s) ||
        h.nx != s->nx || h.ny != s->ny || h.nz != s->nz || h.scheme != s->scheme || h.nclasses != s->nclasses ||
        h.material_hash != s->material_hash || h.steps < 0) {
        std::fclose(f);
        return FDTD_ERR_FORMAT;
    }
    void *ptr[16];
    size_t bytes[16];
    const int nb = state_blocks(s, h.steps, ptr, bytes);
    std::vector<char> buf;
    bool ok = true;
    for (int k = 0; k < nb && ok && st == FDTD_OK; k++) {
        buf.resize(bytes[k]);
        ok = std::fread(buf.data(), 1, bytes[k], f) == bytes[k];
        if (ok)
            st = cu(cudaMemcpy(ptr[k], buf.data(), bytes[k], cudaMemcpyHostToDevice));
    }
    std::fclose(f);
    if (st != FDTD_OK)
        return st;
    if (!ok)
        return FDTD_ERR_FORMAT;
    // with a double-buffered H the other buffer must hold what the step that
    // produced the saved H read (zero where H is never updated); copy it too
    if (s->kernel != FDTD_KERNEL_TWO_PASS)
        for (int c = 0; c < 3 && st == FDTD_OK; c++)
            st = cu(cudaMemcpy(s->h[(h.steps + 1) & 1][c], ptr[c], sizeof(float) * s->ncell,
                               cudaMemcpyDeviceToDevice));
    int steps = h.steps;
    if (st == FDTD_OK)
        st = cu(cudaMemcpy(s->counter, &steps, sizeof(int), cudaMemcpyHostToDevice));
    if (st != FDTD_OK)
        return st;
    s->steps = h.steps;
    s->copy_pending = false;
    s->probe_start = s->steps;
    return FDTD_OK;
}

}  // extern "C"
