// batch.cu -- many independent solves of uneven sizes advanced together.
//
// Each solve keeps its own resident state (H x2, E x2, D x2 or, in a batch of
// the compact form, R x1 -- FP16 residuals and their scale words in the
// 16-bit form -- and the classes) with
// rows padded to a multiple of 16 cells, so every solve gets TMA staging, and
// its own plan (class table, source table, Mur slabs) and step counter.  A
// batched step is three launches: one persistent kernel over the work units
// (column tile x z chunk) of all solves, one Mur launch over all solves' face
// cells, and a one-block kernel that advances the step counters.  Step n of a
// solve uses its counter's parity to pick pointers and tensor maps, so one
// captured graph serves every step; a solve stops once it reaches its target
// step count.  Adding or removing a solve rebuilds the descriptors and the
// graph.  No reference counterpart (the reference runs one grid).
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "native.cuh"

using namespace fdtd;

namespace {

int cu(cudaError_t e) { return e == cudaSuccess ? FDTD_OK : (int)e; }

struct BatchSolve {
    int id = 0;
    int nx = 0, ny = 0, nz = 0, pitch = 0;
    size_t ncell = 0;  // pitch * ny * nz
    size_t bytes = 0;
    int steps_target = 0;
    fdtd_plan *plan = nullptr;
    char *d_block = nullptr;
    float *h[2][3] = {};
    float *e[2][3] = {};
    float *d[2][3] = {};
    uint8_t *mat = nullptr;
    uint32_t *rexp = nullptr;  // 16-bit R form: scale words
    int *counter = nullptr;
};

size_t padded_pitch(int nx) { return ((size_t)nx + 15) & ~size_t(15); }

size_t r16_array_bytes(size_t ncell) { return (ncell * sizeof(uint16_t) + 255) & ~size_t(255); }
size_t r16_exp_bytes(int nx, int ny, int nz) { return (r16_words(nx, ny, nz) * sizeof(uint32_t) + 255) & ~size_t(255); }

size_t state_bytes(int nx, int ny, int nz, bool compact, bool r16 = false)
{
    const size_t ncell = padded_pitch(nx) * ny * nz;
    const size_t f = (ncell * sizeof(float) + 255) & ~size_t(255);
    const size_t d = r16 ? 3 * r16_array_bytes(ncell) + r16_exp_bytes(nx, ny, nz) : (compact ? 3 : 6) * f;
    return 12 * f + d + ((ncell + 255) & ~size_t(255)) + 256;
}

size_t plan_bytes(int nx, int ny, int nz)
{
    // class table, source table, Mur slabs, x-face Mur factors
    return 256 * 32 + 65536 * 4 + 4 * 2 * ((size_t)ny * nz + (size_t)nx * nz + (size_t)nx * ny) +
           16 * 2 * (size_t)ny * nz + 8 * 256 + 256;
}

}  // namespace

struct fdtd_batch {
    int device = 0;
    bool compact = false;  // every solve keeps the compact state
    bool r16 = false;      // ... with R in 16 bits
    cudaStream_t stream = nullptr;
    std::vector<BatchSolve *> solves;
    int next_id = 1;
    bool dirty = true;
    BatchDesc *d_descs = nullptr;
    size_t descs_cap = 0;
    BatchMurBlock *d_mur = nullptr;
    size_t mur_cap = 0;
    int *d_work = nullptr;
    BatchLaunch launch{};
    std::map<int, cudaGraphExec_t> graphs;  // steps per graph -> exec
    size_t bytes = 0;
    int zchunk_max = 0;  // largest z chunk (fdtd_batch_autotune); 0: the form's default
};

namespace {

void free_solve(BatchSolve *v)
{
    if (!v)
        return;
    cudaFree(v->d_block);
    fdtd_plan_destroy(v->plan);
    delete v;
}

void drop_graphs(fdtd_batch *b)
{
    for (auto &kv : b->graphs)
        cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
}

NativeConsts solve_consts(const BatchSolve *v, int parity)
{
    fdtd_native_fields f{};
    const int cur = (parity + 1) & 1, prv = parity & 1;
    for (int k = 0; k < 3; k++) {
        (&f.hx)[k] = v->h[parity][k];
        (&f.hx_out)[k] = v->h[(parity + 1) & 1][k];
        (&f.ex)[k] = v->e[cur][k];
        (&f.ex_prev)[k] = v->e[prv][k];
        (&f.dx)[k] = v->d[cur][k];
        (&f.dx_prev)[k] = v->d[prv][k];
    }
    f.material = v->mat;
    NativeConsts c = make_consts(v->plan, &f, 0);
    c.pitch = v->pitch;
    c.step_counter = v->counter;
    c.r_exp = v->rexp;
    return c;
}

int rebuild(fdtd_batch *b)
{
    std::vector<BatchDesc> descs(b->solves.size());
    std::vector<BatchMurBlock> mur;
    int units = 0;
    const int ty = fused_tile_height();
    for (size_t i = 0; i < b->solves.size(); i++) {
        BatchSolve *v = b->solves[i];
        BatchDesc &d = descs[i];
        std::memset(&d, 0, sizeof d);
        for (int par = 0; par < 2; par++) {
            d.c[par] = solve_consts(v, par);
            if (!encode_step_maps(d.c[par], b->compact, &d.maps[par], b->r16))
                return FDTD_ERR_INVALID;
        }
        d.zchunk = b->zchunk_max > 0 ? zchunk_limited(v->nz, b->zchunk_max)
                                     : (b->compact ? compact_zchunk(v->nz) : fused_zchunk(v->nz));
        d.tiles_x = (v->nx + 31) / 32;
        d.tiles_y = (v->ny + ty - 1) / ty;
        d.chunks = (v->nz + d.zchunk - 1) / d.zchunk;
        d.unit_begin = units;
        d.unit_count = d.tiles_x * d.tiles_y * d.chunks;
        d.steps_target = v->steps_target;
        units += d.unit_count;
        for (int f = 0; f < 12; f++) {
            const MurFace m = mur_face(f, v->nx, v->ny, v->nz);
            const long long cells = (long long)m.len_u * m.len_v;
            for (long long first = 0; first < cells; first += BATCH_MUR_CELLS)
                mur.push_back(BatchMurBlock{(int)i, f, (int)first, 0});
        }
    }
    int st = FDTD_OK;
    if (descs.size() > b->descs_cap) {
        cudaFree(b->d_descs);
        b->d_descs = nullptr;
        st = cu(cudaMalloc(&b->d_descs, sizeof(BatchDesc) * descs.size()));
        b->descs_cap = st == FDTD_OK ? descs.size() : 0;
    }
    if (st == FDTD_OK && mur.size() > b->mur_cap) {
        cudaFree(b->d_mur);
        b->d_mur = nullptr;
        st = cu(cudaMalloc(&b->d_mur, sizeof(BatchMurBlock) * mur.size()));
        b->mur_cap = st == FDTD_OK ? mur.size() : 0;
    }
    if (st == FDTD_OK && !descs.empty())
        st = cu(cudaMemcpyAsync(b->d_descs, descs.data(), sizeof(BatchDesc) * descs.size(), cudaMemcpyHostToDevice,
                                b->stream));
    if (st == FDTD_OK && !mur.empty())
        st = cu(cudaMemcpyAsync(b->d_mur, mur.data(), sizeof(BatchMurBlock) * mur.size(), cudaMemcpyHostToDevice,
                                b->stream));
    if (st == FDTD_OK)
        st = cu(cudaStreamSynchronize(b->stream));
    if (st != FDTD_OK)
        return st;
    int max_classes = 1;
    for (auto *v : b->solves)
        max_classes = std::max(max_classes, v->plan->nclasses);
    b->launch = BatchLaunch{b->d_descs, (int)descs.size(), units, b->d_work, b->d_mur, (int)mur.size(),
                            batch_persistent_ctas(b->compact, max_classes, b->r16), b->compact ? 1 : 0, max_classes,
                            b->r16 ? 1 : 0};
    drop_graphs(b);
    b->dirty = false;
    return FDTD_OK;
}

int graph_for(fdtd_batch *b, int len, cudaGraphExec_t *out)
{
    auto it = b->graphs.find(len);
    if (it != b->graphs.end()) {
        *out = it->second;
        return FDTD_OK;
    }
    int st = cu(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    if (st != FDTD_OK)
        return st;
    for (int k = 0; k < len && st == FDTD_OK; k++)
        st = launch_batch_step(b->launch, b->stream);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (st != FDTD_OK || e != cudaSuccess) {
        if (g)
            cudaGraphDestroy(g);
        return st != FDTD_OK ? st : (int)e;
    }
    cudaGraphExec_t exec = nullptr;
    st = cu(cudaGraphInstantiate(&exec, g, 0));
    cudaGraphDestroy(g);
    if (st != FDTD_OK)
        return st;
    b->graphs[len] = exec;
    *out = exec;
    return FDTD_OK;
}

// Sum over the solves of cells x completed steps (synchronises).
int cell_steps(fdtd_batch *b, double *out)
{
    int st = cu(cudaStreamSynchronize(b->stream));
    double sum = 0.0;
    for (auto *v : b->solves) {
        int n = 0;
        if (st == FDTD_OK)
            st = cu(cudaMemcpy(&n, v->counter, sizeof n, cudaMemcpyDeviceToHost));
        sum += (double)v->nx * v->ny * v->nz * n;
    }
    *out = sum;
    return st;
}

BatchSolve *find(fdtd_batch *b, int id)
{
    for (auto *v : b->solves)
        if (v->id == id)
            return v;
    return nullptr;
}

}  // namespace

extern "C" {

size_t fdtd_batch_solve_bytes(int nx, int ny, int nz)
{
    if (nx < 3 || ny < 3 || nz < 3)
        return 0;
    return state_bytes(nx, ny, nz, false) + plan_bytes(nx, ny, nz);
}

size_t fdtd_batch_need_bytes(const fdtd_batch *b, int nx, int ny, int nz)
{
    if (!b || nx < 3 || ny < 3 || nz < 3)
        return 0;
    return state_bytes(nx, ny, nz, b->compact, b->r16) + plan_bytes(nx, ny, nz);
}

int fdtd_batch_create(int device, fdtd_batch **out) { return fdtd_batch_create_form(device, FDTD_KERNEL_SINGLE_PASS, out); }

int fdtd_batch_create_form(int device, int kernel, fdtd_batch **out)
{
    if (!out || (kernel != FDTD_KERNEL_SINGLE_PASS && kernel != FDTD_KERNEL_COMPACT &&
                 kernel != FDTD_KERNEL_COMPACT_R16))
        return FDTD_ERR_INVALID;
    int st = cu(cudaSetDevice(device));
    if (st != FDTD_OK)
        return st;
    auto *b = new (std::nothrow) fdtd_batch();
    if (!b)
        return FDTD_ERR_NOMEM;
    b->device = device;
    b->compact = kernel == FDTD_KERNEL_COMPACT || kernel == FDTD_KERNEL_COMPACT_R16;
    b->r16 = kernel == FDTD_KERNEL_COMPACT_R16;
    st = cu(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    if (st == FDTD_OK)
        st = cu(cudaMalloc(&b->d_work, 256));
    if (st == FDTD_OK)
        st = cu(cudaMemset(b->d_work, 0, 256));
    if (st != FDTD_OK) {
        fdtd_batch_destroy(b);
        return st;
    }
    *out = b;
    return FDTD_OK;
}

int fdtd_batch_destroy(fdtd_batch *b)
{
    if (!b)
        return FDTD_OK;
    cudaSetDevice(b->device);
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    for (auto *v : b->solves)
        free_solve(v);
    cudaFree(b->d_descs);
    cudaFree(b->d_mur);
    cudaFree(b->d_work);
    if (b->stream)
        cudaStreamDestroy(b->stream);
    delete b;
    return FDTD_OK;
}

int fdtd_batch_add(fdtd_batch *b, const fdtd_solver_config *cfg, int steps, int *id_out)
{
    if (!b || !cfg || !cfg->params || !cfg->material || !cfg->specs || steps < 0 || !id_out)
        return FDTD_ERR_INVALID;
    const FdtdParams *p = cfg->params;
    if (p->nx < 3 || p->ny < 3 || p->nz < 3)
        return FDTD_ERR_INVALID;
    for (int f = 0; f < 12; f++) {  // the Mur block table indexes face cells with 32-bit offsets
        const MurFace m = mur_face(f, p->nx, p->ny, p->nz);
        if ((long long)m.len_u * m.len_v >= (1ll << 31))
            return FDTD_ERR_INVALID;
    }
    int st = cu(cudaSetDevice(b->device));
    if (st == FDTD_OK)
        st = cu(cudaStreamSynchronize(b->stream));
    if (st != FDTD_OK)
        return st;
    if (scan_material(cfg->material, p->nx, p->ny, p->nz, cfg->nclasses, nullptr) != FDTD_OK)
        return FDTD_ERR_INVALID;
    auto *v = new (std::nothrow) BatchSolve();
    if (!v)
        return FDTD_ERR_NOMEM;
    v->nx = p->nx; v->ny = p->ny; v->nz = p->nz;
    v->pitch = (int)padded_pitch(p->nx);
    v->ncell = (size_t)v->pitch * v->ny * v->nz;
    v->steps_target = steps;
    st = fdtd_plan_create(p, cfg->specs, cfg->nclasses, cfg->scheme, nullptr, &v->plan);
    const size_t fbytes = (v->ncell * sizeof(float) + 255) & ~size_t(255);
    const size_t total = state_bytes(p->nx, p->ny, p->nz, b->compact, b->r16);
    const size_t dbytes = b->r16 ? r16_array_bytes(v->ncell) : fbytes;
    if (st == FDTD_OK)
        st = cu(cudaMalloc(&v->d_block, total));
    if (st == FDTD_OK)
        st = cu(cudaMemsetAsync(v->d_block, 0, total, b->stream));
    if (st == FDTD_OK) {
        char *q = v->d_block;
        for (int s = 0; s < 2; s++)
            for (int k = 0; k < 3; k++, q += fbytes)
                v->h[s][k] = reinterpret_cast<float *>(q);
        for (int s = 0; s < 2; s++)
            for (int k = 0; k < 3; k++, q += fbytes)
                v->e[s][k] = reinterpret_cast<float *>(q);
        const int nd = b->compact ? 1 : 2;  // D^n, D^{n-1} slots, or the one R array
        for (int s = 0; s < nd; s++)
            for (int k = 0; k < 3; k++, q += dbytes)
                v->d[s][k] = reinterpret_cast<float *>(q);
        if (nd == 1)
            for (int k = 0; k < 3; k++)
                v->d[1][k] = v->d[0][k];
        if (b->r16) {
            v->rexp = reinterpret_cast<uint32_t *>(q);
            q += r16_exp_bytes(p->nx, p->ny, p->nz);
        }
        v->mat = reinterpret_cast<uint8_t *>(q);
        q += (v->ncell + 255) & ~size_t(255);
        v->counter = reinterpret_cast<int *>(q);
        // dense host classes -> padded rows (one 2-D copy per z plane range)
        st = cu(cudaMemcpy2DAsync(v->mat, v->pitch, cfg->material, p->nx, p->nx, (size_t)p->ny * p->nz,
                                  cudaMemcpyHostToDevice, b->stream));
    }
    if (st == FDTD_OK)
        st = cu(cudaStreamSynchronize(b->stream));
    if (st != FDTD_OK) {
        free_solve(v);
        return st;
    }
    v->bytes = total + plan_bytes(p->nx, p->ny, p->nz);
    v->id = b->next_id++;
    b->solves.push_back(v);
    b->bytes += v->bytes;
    b->dirty = true;
    *id_out = v->id;
    return FDTD_OK;
}

int fdtd_batch_remove(fdtd_batch *b, int id)
{
    if (!b)
        return FDTD_ERR_INVALID;
    BatchSolve *v = find(b, id);
    if (!v)
        return FDTD_ERR_INVALID;
    cudaSetDevice(b->device);
    const int st = cu(cudaStreamSynchronize(b->stream));
    b->solves.erase(std::find(b->solves.begin(), b->solves.end(), v));
    b->bytes -= v->bytes;
    free_solve(v);
    b->dirty = true;
    return st;
}

int fdtd_batch_run(fdtd_batch *b, int nsteps)
{
    if (!b || nsteps < 0)
        return FDTD_ERR_INVALID;
    int st = cu(cudaSetDevice(b->device));
    if (st != FDTD_OK || nsteps == 0 || b->solves.empty())
        return st;
    if (b->dirty && (st = rebuild(b)) != FDTD_OK)
        return st;
    const int chunk = 8;
    while (nsteps > 0 && st == FDTD_OK) {
        const int len = nsteps >= chunk ? chunk : 1;
        cudaGraphExec_t g;
        st = graph_for(b, len, &g);
        if (st == FDTD_OK)
            st = cu(cudaGraphLaunch(g, b->stream));
        nsteps -= len;
    }
    return st;
}

int fdtd_batch_autotune(fdtd_batch *b, int steps_per_trial, int *chosen)
{
    if (!b || steps_per_trial < 1)
        return FDTD_ERR_INVALID;
    int st = cu(cudaSetDevice(b->device));
    if (st != FDTD_OK)
        return st;
    // D form: at most 64 planes (the per-thread source-plane mask covers 66)
    static const int compact_cands[] = {8, 12, 16, 24, 32, 48, 64};
    static const int dform_cands[] = {16, 24, 32, 48, 64};
    const int *cands = b->compact ? compact_cands : dform_cands;
    const int ncand = b->compact ? 7 : 5;
    const int trial = (steps_per_trial + 7) / 8 * 8;  // whole 8-step graphs only
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    st = cu(cudaEventCreate(&e0));
    if (st == FDTD_OK)
        st = cu(cudaEventCreate(&e1));
    double best_cost = 0.0;
    int best = 0;
    for (int k = 0; k < ncand && st == FDTD_OK && !b->solves.empty(); k++) {
        b->zchunk_max = cands[k];
        b->dirty = true;
        st = fdtd_batch_run(b, 8);  // rebuild and graph capture, untimed
        double c0 = 0.0, c1 = 0.0;
        if (st == FDTD_OK)
            st = cell_steps(b, &c0);
        if (st == FDTD_OK)
            st = cu(cudaEventRecord(e0, b->stream));
        if (st == FDTD_OK)
            st = fdtd_batch_run(b, trial);
        if (st == FDTD_OK)
            st = cu(cudaEventRecord(e1, b->stream));
        if (st == FDTD_OK)
            st = cell_steps(b, &c1);
        float ms = 0.0f;
        if (st == FDTD_OK)
            st = cu(cudaEventElapsedTime(&ms, e0, e1));
        if (st == FDTD_OK && c1 > c0) {
            const double cost = ms / (c1 - c0);
            if (best == 0 || cost < best_cost) {
                best_cost = cost;
                best = cands[k];
            }
        }
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    b->zchunk_max = best;  // 0 when no trial advanced a solve: the default
    b->dirty = true;
    if (chosen)
        *chosen = best;
    if (st == FDTD_OK)
        st = fdtd_batch_synchronize(b);
    return st;
}

int fdtd_batch_synchronize(fdtd_batch *b)
{
    if (!b)
        return FDTD_ERR_INVALID;
    cudaSetDevice(b->device);
    int st = cu(cudaStreamSynchronize(b->stream));
    for (auto *v : b->solves)
        if (st == FDTD_OK)
            st = plan_error(v->plan);
    return st;
}

int fdtd_batch_steps(fdtd_batch *b, int id)
{
    if (!b)
        return -1;
    BatchSolve *v = find(b, id);
    if (!v || fdtd_batch_synchronize(b) != FDTD_OK)
        return -1;
    int n = -1;
    if (cudaMemcpy(&n, v->counter, sizeof n, cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
    return n;
}

int fdtd_batch_get_field(fdtd_batch *b, int id, int field, int z0, int nplanes, float *host_out)
{
    if (!b || !host_out || field < 0 || field >= FDTD_FIELD_COUNT)
        return FDTD_ERR_INVALID;
    BatchSolve *v = find(b, id);
    if (!v)
        return FDTD_ERR_INVALID;
    if (nplanes == 0) {
        z0 = 0;
        nplanes = v->nz;
    }
    if (z0 < 0 || nplanes < 0 || z0 + nplanes > v->nz)
        return FDTD_ERR_INVALID;
    if (b->compact && field >= FDTD_FIELD_DX && field <= FDTD_FIELD_DZ)
        return FDTD_ERR_INVALID;  // D is not stored
    int st = fdtd_batch_synchronize(b);
    int n = 0;
    if (st == FDTD_OK)
        st = cu(cudaMemcpy(&n, v->counter, sizeof n, cudaMemcpyDeviceToHost));
    if (st != FDTD_OK)
        return st;
    const int comp = field % 3;
    const float *src;
    if (field < 3)
        src = v->h[n & 1][comp];
    else {
        const int slot = n > 0 ? ((n - 1) & 1) : 0;
        src = field < 6 ? v->d[slot][comp] : v->e[slot][comp];
    }
    src += (size_t)z0 * v->pitch * v->ny;
    return cu(cudaMemcpy2D(host_out, sizeof(float) * v->nx, src, sizeof(float) * v->pitch, sizeof(float) * v->nx,
                           (size_t)v->ny * nplanes, cudaMemcpyDeviceToHost));
}

size_t fdtd_batch_bytes(const fdtd_batch *b) { return b ? b->bytes : 0; }

int fdtd_batch_size(const fdtd_batch *b) { return b ? (int)b->solves.size() : 0; }

fdtd_stream_t fdtd_batch_stream(const fdtd_batch *b) { return b ? b->stream : nullptr; }

}  // extern "C"
