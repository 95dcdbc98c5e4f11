// batch.cu -- many independent solves of uneven sizes advanced together.
//
// Each solve keeps its own resident state (H x2, E x2, D x2 or, in a batch of
// the compact form, R x1 -- FP16 residuals and their scale words in the
// 16-bit form -- and the classes) with
// rows padded to a multiple of 16 cells, so every solve gets TMA staging, and
// its own plan (class table, source table, Mur slabs) and step counter.  A
// batched step is three launches: one kernel over the work units (column
// tile x z chunk) of all solves (compact forms: one CTA per unit; D form: a
// persistent kernel taking units from a counter), one Mur launch over all solves' face
// cells, and a one-block kernel that advances the step counters.  Step n of a
// solve uses its counter's parity to pick pointers and tensor maps, so one
// captured graph serves every step; a solve stops once it reaches its target
// step count.  Adding or removing a solve rebuilds the descriptors and the
// graph.  No reference counterpart (the reference runs one grid).
//
// Nothing on the way of a running batch waits for the GPU: a new solve's
// memory comes from the batch's stream-ordered pool and its uploads run on a
// side stream (the batch stream waits for them before the solve's first
// step); descriptor uploads go through pinned staging buffers; a removed
// solve's memory is freed in stream order behind the work that reads it; and
// field reads can be queued as copies into the caller's host memory, with a
// ticket to poll.  A serving loop can so admit, snapshot and retire solves
// while earlier batched steps still run.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>

#include "native.cuh"
#include "strip_unit.cuh"

using namespace fdtd;

namespace {
constexpr int STRIP_SHAPE_COUNT = strip::STRIP_SHAPES;
}

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
    int host_steps = 0;              // steps queued for this solve so far (its counter once they ran)
    cudaEvent_t ready = nullptr;     // its uploads on the side stream; waited for before its first step
    std::vector<unsigned char> memless8;  // compact forms: tile-planes (32 x 8) without Debye memory
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

// Pinned host buffer for descriptor uploads; done marks the end of its last upload.
struct StageBuf {
    void *host = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
};

struct fdtd_batch {
    int device = 0;
    bool compact = false;  // every solve keeps the compact state
    bool r16 = false;      // ... with R in 16 bits
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;      // uploads of solves being added
    cudaMemPool_t pool = nullptr;     // device memory of the solves, descriptors and Mur blocks
    StageBuf stage[2];                // alternating pinned staging of descriptor uploads
    int stage_next = 0;
    std::vector<cudaEvent_t> spare_events;
    std::map<long long, cudaEvent_t> tickets;  // queued reads and marks
    long long next_ticket = 1;
    bool timing = false;              // events around every fdtd_batch_run (busy time)
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> runs;
    double busy_ms = 0.0, span_ms = 0.0;
    cudaEvent_t first_start = nullptr;
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
    int strip_shape = 0;  // compact forms: strip kernel shape, -1 the z-marching kernel (fdtd_batch_autotune)
    bool strip = false;   // the current launch runs the strip kernel
    BatchUnit *d_units = nullptr;  // strip kernel: per unit its solve and memoryless planes
    size_t units_cap = 0;
};

namespace {

// Frees a solve in stream order on s (behind the work queued there).
void free_solve(BatchSolve *v, cudaStream_t s)
{
    if (!v)
        return;
    if (v->d_block)
        cudaFreeAsync(v->d_block, s);
    plan_destroy_on(v->plan, s);
    if (v->ready)
        cudaEventDestroy(v->ready);
    delete v;
}

cudaEvent_t take_event(fdtd_batch *b)
{
    if (!b->spare_events.empty()) {
        cudaEvent_t e = b->spare_events.back();
        b->spare_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    return cudaEventCreate(&e) == cudaSuccess ? e : nullptr;
}

// Device memory from the batch's pool, in stream order on s.
int pool_alloc(fdtd_batch *b, void **p, size_t bytes, cudaStream_t s)
{
    return cu(cudaMallocFromPoolAsync(p, bytes, b->pool, s));
}

// One host -> device copy of a table upload.
struct Upload {
    void *dst;
    const void *src;
    size_t n;
};

// Copies the tables of one rebuild to the device on the batch stream through
// the next pinned staging buffer, all in one buffer, so that a rebuild waits
// only for the upload of the rebuild before the previous one (the buffer's
// last use), not for the steps queued since.
int staged_upload(fdtd_batch *b, const std::vector<Upload> &ups)
{
    size_t total = 0;
    for (const Upload &u : ups)
        total += (u.n + 15) & ~size_t(15);
    if (total == 0)
        return FDTD_OK;
    StageBuf &sb = b->stage[b->stage_next];
    b->stage_next ^= 1;
    int st = cu(cudaEventSynchronize(sb.done));
    if (st == FDTD_OK && sb.cap < total) {
        if (sb.host)
            cudaFreeHost(sb.host);
        sb.host = nullptr;
        sb.cap = 0;
        const size_t cap = std::max(total, size_t(1) << 20);
        st = cu(cudaHostAlloc(&sb.host, cap, cudaHostAllocDefault));
        if (st == FDTD_OK)
            sb.cap = cap;
    }
    size_t off = 0;
    for (const Upload &u : ups) {
        if (st != FDTD_OK || u.n == 0)
            continue;
        unsigned char *h = static_cast<unsigned char *>(sb.host) + off;
        std::memcpy(h, u.src, u.n);
        st = cu(cudaMemcpyAsync(u.dst, h, u.n, cudaMemcpyHostToDevice, b->stream));
        off += (u.n + 15) & ~size_t(15);
    }
    if (st == FDTD_OK)
        st = cu(cudaEventRecord(sb.done, b->stream));
    return st;
}

// Busy time of the completed timed runs (in order), added to b's totals.
void collect_runs(fdtd_batch *b)
{
    size_t k = 0;
    for (; k < b->runs.size(); k++) {
        auto &r = b->runs[k];
        if (cudaEventQuery(r.second) != cudaSuccess)
            break;
        float ms = 0.0f, span = 0.0f;
        cudaEventElapsedTime(&ms, r.first, r.second);
        b->busy_ms += ms;
        cudaEventElapsedTime(&span, b->first_start, r.second);
        b->span_ms = span;
        if (r.first != b->first_start)
            b->spare_events.push_back(r.first);
        b->spare_events.push_back(r.second);
    }
    b->runs.erase(b->runs.begin(), b->runs.begin() + k);
}

void drop_graphs(fdtd_batch *b)
{
    for (auto &kv : b->graphs)
        cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
}

NativeConsts solve_consts(const BatchSolve *v, int parity, int *err)
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
    c.err = err;  // one error word for the batch
    return c;
}

// Word of the batch's work buffer that a bounded wait which gave up sets.
constexpr int BATCH_ERR_WORD = 32;

int rebuild(fdtd_batch *b)
{
    std::vector<BatchDesc> descs(b->solves.size());
    std::vector<BatchMurBlock> mur;
    int units = 0;
    // compact forms run the strip kernel when every solve's arrays are
    // TMA-addressable for it (and the autotuner did not choose the
    // z-marching kernel: shape -1), else the z-marching kernel
    bool strip = b->compact && b->strip_shape >= 0;
    for (auto *v : b->solves)
        if (strip) {
            NativeConsts c = solve_consts(v, 0, b->d_work + BATCH_ERR_WORD);
            strip = strip_usable(c, b->r16);
        }
    const int ty = strip ? strip_shape_rows(b->strip_shape) : fused_tile_height();
    for (size_t i = 0; i < b->solves.size(); i++) {
        BatchSolve *v = b->solves[i];
        BatchDesc &d = descs[i];
        std::memset(&d, 0, sizeof d);
        for (int par = 0; par < 2; par++) {
            d.c[par] = solve_consts(v, par, b->d_work + BATCH_ERR_WORD);
            d.c[par].fuse_mur_x = strip ? 1 : 0;  // the strip kernel applies the x-face Mur updates
            if (strip ? !strip::encode_strip_maps(d.c[par], b->r16, ty, &d.smaps[par])
                      : !encode_step_maps(d.c[par], b->compact, &d.maps[par], b->r16))
                return FDTD_ERR_INVALID;
        }
        d.zchunk = b->zchunk_max > 0 ? zchunk_limited(v->nz, b->zchunk_max)
                                     : (strip ? strip_zchunk(v->nz)
                                              : (b->compact ? compact_zchunk(v->nz) : fused_zchunk(v->nz)));
        d.tiles_x = (v->nx + 31) / 32;
        d.tiles_y = (v->ny + ty - 1) / ty;
        d.chunks = (v->nz + d.zchunk - 1) / d.zchunk;
        d.unit_begin = units;
        d.unit_count = d.tiles_x * d.tiles_y * d.chunks;
        d.steps_target = v->steps_target;
        units += d.unit_count;
        const int fused = mur_x_fused_faces(d.c[0]);
        for (int f = 0; f < 12; f++) {
            const MurFace m = mur_face(f, v->nx, v->ny, v->nz);
            long long cells = (long long)m.len_u * m.len_v;
            int limit = 0;
            if (m.axis == 0 && (fused & (m.far ? 2 : 1))) {
                if (m.comp == 1)
                    continue;  // ey x face: updated by the step kernel
                cells = m.len_u;  // ez x face: only the z = 0 row is left
                limit = m.len_u;
            }
            for (long long first = 0; first < cells; first += BATCH_MUR_CELLS)
                mur.push_back(BatchMurBlock{(int)i, f, (int)first, limit});
        }
    }
    // new solves: the batch stream waits for their uploads on the side stream
    int st = FDTD_OK;
    for (auto *v : b->solves)
        if (v->ready && st == FDTD_OK) {
            st = cu(cudaStreamWaitEvent(b->stream, v->ready, 0));
            cudaEventDestroy(v->ready);
            v->ready = nullptr;
        }
    // device tables grow in stream order (the old ones are freed behind the
    // steps that still read them)
    if (st == FDTD_OK && descs.size() > b->descs_cap) {
        if (b->d_descs)
            cudaFreeAsync(b->d_descs, b->stream);
        b->d_descs = nullptr;
        const size_t cap = std::max(descs.size() * 2, size_t(16));
        st = pool_alloc(b, reinterpret_cast<void **>(&b->d_descs), sizeof(BatchDesc) * cap, b->stream);
        b->descs_cap = st == FDTD_OK ? cap : 0;
    }
    if (st == FDTD_OK && mur.size() > b->mur_cap) {
        if (b->d_mur)
            cudaFreeAsync(b->d_mur, b->stream);
        b->d_mur = nullptr;
        const size_t cap = std::max(mur.size() * 2, size_t(1024));
        st = pool_alloc(b, reinterpret_cast<void **>(&b->d_mur), sizeof(BatchMurBlock) * cap, b->stream);
        b->mur_cap = st == FDTD_OK ? cap : 0;
    }
    // strip kernel: per unit its tile, z chunk, solve and the planes whose
    // tile holds no Debye memory
    std::vector<BatchUnit> recs;
    if (strip) {
        std::vector<unsigned long long> masks((size_t)units, 0ull);
        recs.resize((size_t)units);
        for (size_t i = 0; i < b->solves.size(); i++) {
            const BatchSolve *v = b->solves[i];
            const BatchDesc &d = descs[i];
            if (d.tiles_x > 65535 || d.tiles_y > 65535 || d.chunks > 65535 || d.zchunk > 65535)
                return FDTD_ERR_INVALID;
            strip_unit_masks(v->memless8, v->nx, v->ny, v->nz, ty, d.zchunk, masks.data() + d.unit_begin);
            for (int j = 0; j < d.unit_count; j++) {
                const int per_z = d.tiles_x * d.tiles_y, rem = j % per_z;
                recs[(size_t)d.unit_begin + j] =
                    BatchUnit{masks[(size_t)d.unit_begin + j], v->counter,           (int)i,
                              (unsigned short)(rem % d.tiles_x), (unsigned short)(rem / d.tiles_x),
                              (unsigned short)(j / per_z),       (unsigned short)d.zchunk, d.steps_target};
            }
        }
        if (st == FDTD_OK && recs.size() > b->units_cap) {
            if (b->d_units)
                cudaFreeAsync(b->d_units, b->stream);
            b->d_units = nullptr;
            const size_t cap = std::max(recs.size() * 2, size_t(1024));
            st = pool_alloc(b, reinterpret_cast<void **>(&b->d_units), sizeof(BatchUnit) * cap, b->stream);
            b->units_cap = st == FDTD_OK ? cap : 0;
        }
    }
    if (st == FDTD_OK)
        st = staged_upload(b, {Upload{b->d_descs, descs.data(), sizeof(BatchDesc) * descs.size()},
                               Upload{b->d_mur, mur.data(), sizeof(BatchMurBlock) * mur.size()},
                               Upload{b->d_units, recs.data(), sizeof(BatchUnit) * recs.size()}});
    if (st != FDTD_OK)
        return st;
    int max_classes = 1;
    for (auto *v : b->solves)
        max_classes = std::max(max_classes, v->plan->nclasses);
    const int ctas = strip ? batch_strip_ctas(b->r16, b->strip_shape, max_classes)
                           : batch_persistent_ctas(b->compact, max_classes, b->r16);
    if (ctas < 1)
        return FDTD_ERR_INVALID;
    b->launch = BatchLaunch{b->d_descs, (int)descs.size(), units, b->d_work, b->d_mur, (int)mur.size(), ctas,
                            b->compact ? 1 : 0, max_classes, b->r16 ? 1 : 0, strip ? 1 : 0, b->strip_shape,
                            strip ? b->d_units : nullptr};
    b->strip = strip;
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
        st = cu(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
    if (st == FDTD_OK) {
        // the batch's own pool keeps freed memory for the next solves
        // instead of handing it back to CUDA
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        st = cu(cudaMemPoolCreate(&b->pool, &props));
        if (st == FDTD_OK) {
            uint64_t keep = UINT64_MAX;
            st = cu(cudaMemPoolSetAttribute(b->pool, cudaMemPoolAttrReleaseThreshold, &keep));
        }
    }
    for (int k = 0; k < 2 && st == FDTD_OK; k++)
        st = cu(cudaEventCreateWithFlags(&b->stage[k].done, cudaEventDisableTiming));
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
    if (b->side)
        cudaStreamSynchronize(b->side);
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    cudaStream_t s = b->stream ? b->stream : b->side;
    for (auto *v : b->solves)
        free_solve(v, s);
    if (b->d_descs)
        cudaFreeAsync(b->d_descs, s);
    if (b->d_mur)
        cudaFreeAsync(b->d_mur, s);
    if (b->d_units)
        cudaFreeAsync(b->d_units, s);
    if (s)
        cudaStreamSynchronize(s);
    cudaFree(b->d_work);
    for (auto &sb : b->stage) {
        if (sb.host)
            cudaFreeHost(sb.host);
        if (sb.done)
            cudaEventDestroy(sb.done);
    }
    for (auto &kv : b->tickets)
        cudaEventDestroy(kv.second);
    for (auto &r : b->runs) {
        if (r.first != b->first_start)
            cudaEventDestroy(r.first);
        cudaEventDestroy(r.second);
    }
    if (b->first_start)
        cudaEventDestroy(b->first_start);
    for (auto e : b->spare_events)
        cudaEventDestroy(e);
    if (b->pool)
        cudaMemPoolDestroy(b->pool);
    if (b->side)
        cudaStreamDestroy(b->side);
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
    if (st != FDTD_OK)
        return st;
    if (cfg->nclasses < 1 || cfg->nclasses > FDTD_MAX_CLASSES)
        return FDTD_ERR_INVALID;
    int top = 0;
    if (scan_material(cfg->material, p->nx, p->ny, p->nz, cfg->nclasses, nullptr, &top) != FDTD_OK)
        return FDTD_ERR_INVALID;
    const int ncls = top + 1;  // the classes up to the largest one present
    auto *v = new (std::nothrow) BatchSolve();
    if (!v)
        return FDTD_ERR_NOMEM;
    v->nx = p->nx; v->ny = p->ny; v->nz = p->nz;
    v->pitch = (int)padded_pitch(p->nx);
    v->ncell = (size_t)v->pitch * v->ny * v->nz;
    v->steps_target = steps;
    // everything of the new solve goes on the side stream: the batch stream
    // keeps running the steps already queued
    st = plan_create_on(p, cfg->specs, ncls, cfg->scheme, nullptr, b->pool, b->side, &v->plan);
    const size_t fbytes = (v->ncell * sizeof(float) + 255) & ~size_t(255);
    const size_t total = state_bytes(p->nx, p->ny, p->nz, b->compact, b->r16);
    const size_t dbytes = b->r16 ? r16_array_bytes(v->ncell) : fbytes;
    if (st == FDTD_OK)
        st = pool_alloc(b, reinterpret_cast<void **>(&v->d_block), total, b->side);
    if (st == FDTD_OK)
        st = cu(cudaMemsetAsync(v->d_block, 0, total, b->side));
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
                                  cudaMemcpyHostToDevice, b->side));
    }
    if (st == FDTD_OK)
        st = cu(cudaEventCreateWithFlags(&v->ready, cudaEventDisableTiming));
    if (st == FDTD_OK)
        st = cu(cudaEventRecord(v->ready, b->side));
    // the caller's class volume may go once the copy has read it
    if (st == FDTD_OK)
        st = cu(cudaStreamSynchronize(b->side));
    if (st != FDTD_OK) {
        free_solve(v, b->side);
        return st;
    }
    if (b->compact)
        v->memless8 = strip_plane_flags(cfg->material, p->nx, p->ny, p->nz, p->nx, cfg->specs, ncls);
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
    const int st = cu(cudaSetDevice(b->device));
    b->solves.erase(std::find(b->solves.begin(), b->solves.end(), v));
    b->bytes -= v->bytes;
    if (v->ready) {  // never stepped: its uploads are ordered before the free
        cudaStreamWaitEvent(b->stream, v->ready, 0);
    }
    free_solve(v, b->stream);  // behind the queued steps and reads
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
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (b->timing) {
        t0 = b->first_start ? take_event(b) : nullptr;
        if (!b->first_start) {
            st = cu(cudaEventCreate(&b->first_start));
            t0 = b->first_start;
        }
        t1 = take_event(b);
        if (st == FDTD_OK && (!t0 || !t1))
            st = FDTD_ERR_NOMEM;
        if (st == FDTD_OK)
            st = cu(cudaEventRecord(t0, b->stream));
    }
    const int chunk = 8;
    const int total = nsteps;
    while (nsteps > 0 && st == FDTD_OK) {
        const int len = nsteps >= chunk ? chunk : 1;
        cudaGraphExec_t g;
        st = graph_for(b, len, &g);
        if (st == FDTD_OK)
            st = cu(cudaGraphLaunch(g, b->stream));
        nsteps -= len;
    }
    if (b->timing && st == FDTD_OK) {
        st = cu(cudaEventRecord(t1, b->stream));
        if (st == FDTD_OK)
            b->runs.emplace_back(t0, t1);
    }
    if (st == FDTD_OK)
        for (auto *v : b->solves)
            v->host_steps = std::min(v->steps_target, v->host_steps + total);
    return st;
}

int fdtd_batch_autotune(fdtd_batch *b, int steps_per_trial, int *chosen)
{
    if (!b || steps_per_trial < 1)
        return FDTD_ERR_INVALID;
    int st = cu(cudaSetDevice(b->device));
    if (st != FDTD_OK)
        return st;
    // D form: at most 64 planes (the per-thread source-plane mask covers 66);
    // compact forms: every strip tile shape with each chunk limit (the
    // z-marching kernel, where the strip kernel cannot run, takes shape 0's
    // trials)
    static const int compact_cands[] = {8, 16, 32, 64};
    static const int dform_cands[] = {16, 24, 32, 48, 64};
    const int nz_cand = b->compact ? 4 : 5;
    const int nshape = b->compact ? STRIP_SHAPE_COUNT + 1 : 1;  // strip shapes, then the z-marching kernel
    const int ncand = nz_cand * nshape;
    const int trial = (steps_per_trial + 7) / 8 * 8;  // whole 8-step graphs only
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    st = cu(cudaEventCreate(&e0));
    if (st == FDTD_OK)
        st = cu(cudaEventCreate(&e1));
    double best_cost = 0.0;
    int best = 0, best_shape = b->strip_shape;
    for (int k = 0; k < ncand && st == FDTD_OK && !b->solves.empty(); k++) {
        const int zc = b->compact ? compact_cands[k % nz_cand] : dform_cands[k % nz_cand];
        b->zchunk_max = zc;
        b->strip_shape = k / nz_cand < STRIP_SHAPE_COUNT ? k / nz_cand : -1;
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
                best = zc;
                best_shape = b->strip_shape;
            }
        }
    }
    b->strip_shape = best_shape;
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
    int flag = 0;
    if (st == FDTD_OK)
        st = cu(cudaMemcpy(&flag, b->d_work + BATCH_ERR_WORD, sizeof flag, cudaMemcpyDeviceToHost));
    if (st == FDTD_OK && flag) {
        cudaMemset(b->d_work + BATCH_ERR_WORD, 0, sizeof flag);
        st = FDTD_ERR_DEVICE_TIMEOUT;
    }
    if (b->timing)
        collect_runs(b);
    return st;
}

int fdtd_batch_read_async(fdtd_batch *b, int id, int field, int z0, int nplanes, float *host_out,
                          long long *ticket)
{
    if (!b || !host_out || !ticket || field < 0 || field >= FDTD_FIELD_COUNT)
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
    int st = cu(cudaSetDevice(b->device));
    if (st != FDTD_OK)
        return st;
    if (v->ready) {  // queued before the solve's first step: its uploads come first
        st = cu(cudaStreamWaitEvent(b->stream, v->ready, 0));
        if (st != FDTD_OK)
            return st;
    }
    // the slots as they are after the steps queued so far
    const int n = v->host_steps, comp = field % 3;
    const float *src;
    if (field < 3)
        src = v->h[n & 1][comp];
    else {
        const int slot = n > 0 ? ((n - 1) & 1) : 0;
        src = field < 6 ? v->d[slot][comp] : v->e[slot][comp];
    }
    src += (size_t)z0 * v->pitch * v->ny;
    st = cu(cudaMemcpy2DAsync(host_out, sizeof(float) * v->nx, src, sizeof(float) * v->pitch, sizeof(float) * v->nx,
                              (size_t)v->ny * nplanes, cudaMemcpyDeviceToHost, b->stream));
    if (st != FDTD_OK)
        return st;
    return fdtd_batch_mark(b, ticket);
}

int fdtd_batch_mark(fdtd_batch *b, long long *ticket)
{
    if (!b || !ticket)
        return FDTD_ERR_INVALID;
    cudaSetDevice(b->device);
    cudaEvent_t e = take_event(b);
    if (!e)
        return FDTD_ERR_NOMEM;
    const int st = cu(cudaEventRecord(e, b->stream));
    if (st != FDTD_OK) {
        b->spare_events.push_back(e);
        return st;
    }
    *ticket = b->next_ticket++;
    b->tickets[*ticket] = e;
    return FDTD_OK;
}

int fdtd_batch_ticket(fdtd_batch *b, long long ticket, int wait)
{
    if (!b)
        return FDTD_ERR_INVALID;
    auto it = b->tickets.find(ticket);
    if (it == b->tickets.end())
        return FDTD_ERR_INVALID;
    cudaSetDevice(b->device);
    const cudaError_t e = wait ? cudaEventSynchronize(it->second) : cudaEventQuery(it->second);
    if (e == cudaErrorNotReady)
        return FDTD_ERR_BUSY;
    b->spare_events.push_back(it->second);
    b->tickets.erase(it);
    if (b->timing)
        collect_runs(b);
    return cu(e);
}

int fdtd_batch_set_timing(fdtd_batch *b, int on)
{
    if (!b)
        return FDTD_ERR_INVALID;
    b->timing = on != 0;
    return FDTD_OK;
}

int fdtd_batch_busy(fdtd_batch *b, double *busy_ms, double *span_ms)
{
    if (!b || !busy_ms || !span_ms)
        return FDTD_ERR_INVALID;
    cudaSetDevice(b->device);
    collect_runs(b);
    *busy_ms = b->busy_ms;
    *span_ms = b->span_ms;
    return FDTD_OK;
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

int fdtd_batch_tuning(const fdtd_batch *b, int *zchunk_max, int *tile_rows, int *strip_kernel)
{
    if (!b)
        return FDTD_ERR_INVALID;
    if (zchunk_max)
        *zchunk_max = b->zchunk_max;
    if (tile_rows)
        *tile_rows = b->compact && b->strip_shape >= 0 ? strip_shape_rows(b->strip_shape) : fused_tile_height();
    if (strip_kernel)
        *strip_kernel = b->compact ? b->strip_shape : -1;
    return FDTD_OK;
}

size_t fdtd_batch_bytes(const fdtd_batch *b) { return b ? b->bytes : 0; }

int fdtd_batch_size(const fdtd_batch *b) { return b ? (int)b->solves.size() : 0; }

fdtd_stream_t fdtd_batch_stream(const fdtd_batch *b) { return b ? b->stream : nullptr; }

}  // extern "C"
