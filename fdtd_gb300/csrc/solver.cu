// solver.cu -- solver handle: resident device state, graph-captured step
// loop, snapshots through a pinned ring on a side stream.
//
// Replaces the reference's time loop (fdtd.cu:115-530).  The reference chains
// three streams with events and spawns copy/writer pthreads per step; here one
// compute stream replays CUDA graphs of whole steps, a device counter supplies
// the step index to the kernels, and snapshot copies run on a second stream
// that overlaps the following step.
#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "solver_internal.cuh"

using namespace fdtd;

namespace fdtd {

// Pointers of step n (see native.cu for the slot convention).
fdtd_native_fields step_fields(const fdtd_solver *s, int n)
{
    fdtd_native_fields f{};
    const int cur = (n + 1) & 1, prv = n & 1;
    // single-pass kernels read H from one buffer and write the other
    const bool hdb = s->kernel != FDTD_KERNEL_TWO_PASS;
    const int hin = hdb ? (n & 1) : 0;
    const int hout = hdb ? ((n + 1) & 1) : 0;
    for (int k = 0; k < 3; k++) {
        (&f.hx)[k] = s->h[hin][k];
        (&f.hx_out)[k] = s->h[hout][k];
        (&f.ex)[k] = s->e[cur][k];
        (&f.ex_prev)[k] = s->e[prv][k];
        (&f.dx)[k] = s->d[cur][k];
        (&f.dx_prev)[k] = s->d[prv][k];
    }
    f.material = s->mat;
    return f;
}

NativeConsts solver_consts(const fdtd_solver *s, int n)
{
    const fdtd_native_fields f = step_fields(s, n);
    NativeConsts c = make_consts(s->plan, &f, n);
    c.r_exp = s->rexp;
    c.memless = s->d_memless;
    c.memless_rows = s->memless_rows;
    return c;
}

// Device buffer holding `field` after `count` completed steps.
const float *field_buffer(const fdtd_solver *s, int field, int count)
{
    const int comp = field % 3;
    if (field < 3) {
        const int idx = s->kernel != FDTD_KERNEL_TWO_PASS ? (count & 1) : 0;
        return s->h[idx][comp];
    }
    if (field < 6 && stores_no_d(s->kernel))
        return nullptr;  // D is not stored
    // E^{count}, D^{count} live in slot (count - 1) % 2; before any step both slots are zero.
    const int slot = count > 0 ? ((count - 1) & 1) : 0;
    return field < 6 ? s->d[slot][comp] : s->e[slot][comp];
}

void reset_graphs(fdtd_solver *s)
{
    for (auto &kv : s->graphs)
        cudaGraphExecDestroy(kv.second);
    s->graphs.clear();
}

}  // namespace fdtd

namespace {

int cu(cudaError_t e) { return e == cudaSuccess ? FDTD_OK : (int)e; }

int enqueue_step(fdtd_solver *s, int n)
{
    NativeConsts c = solver_consts(s, n);
    c.step_counter = s->counter;
    // in a graph the step's first kernel follows the previous step's Mur
    // kernel unless a monitor kernel runs between them
    c.overlap_prev = s->nprobes == 0 && !s->dft_on;
    int st;
    if (s->kernel == FDTD_KERNEL_SINGLE_PASS) {
        st = launch_step(c, s->stream);
    } else if (s->kernel == FDTD_KERNEL_COMPACT) {
        st = launch_step_compact(c, s->stream);
    } else if (s->kernel == FDTD_KERNEL_COMPACT_R16) {
        st = launch_step_compact16(c, s->stream);
    } else {
        st = launch_h(c, s->stream);
        if (st == FDTD_OK)
            st = launch_de(c, s->stream);
        if (st == FDTD_OK)
            st = launch_mur(c, s->stream);
    }
    if (st == FDTD_OK)
        st = launch_monitor(s, n);
    return st;
}

int get_graph(fdtd_solver *s, int parity, int len, cudaGraphExec_t *out)
{
    auto key = std::make_pair(parity, len);
    auto it = s->graphs.find(key);
    if (it != s->graphs.end()) {
        *out = it->second;
        return FDTD_OK;
    }
    cudaGraph_t g = nullptr;
    int st = cu(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    if (st != FDTD_OK)
        return st;
    for (int k = 0; k < len && st == FDTD_OK; k++)
        st = enqueue_step(s, parity + k);  // only the parity of n matters for the pointers
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (st != FDTD_OK) {
        if (g)
            cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess)
        return e;
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
        return e;
    s->graphs[key] = exec;
    *out = exec;
    return FDTD_OK;
}

// Launch `len` consecutive steps starting at s->steps.
int launch_steps(fdtd_solver *s, int len)
{
    // Graph length: long chunks for small grids (launch-bound), short ones
    // for large grids.
    const int chunk = s->ncell >= (size_t(1) << 24) ? 2 : 16;
    while (len > 0) {
        if (s->copy_pending && s->steps >= s->copy_step + s->copy_gap) {
            int st = cu(cudaStreamWaitEvent(s->stream, s->ev_copy, 0));
            if (st != FDTD_OK)
                return st;
            s->copy_pending = false;
        }
        int l = std::min(len, chunk);
        // A pending snapshot copy must finish before step copy_step + copy_gap.
        if (s->copy_pending)
            l = std::min(l, s->copy_step + s->copy_gap - s->steps);
        if (l != chunk)
            l = 1;
        cudaGraphExec_t g;
        int st = get_graph(s, s->steps & 1, l, &g);
        if (st != FDTD_OK)
            return st;
        st = cu(cudaGraphLaunch(g, s->stream));
        if (st != FDTD_OK)
            return st;
        s->steps += l;
        len -= l;
    }
    return FDTD_OK;
}

void CUDART_CB snapshot_ready(void *arg)
{
    // Runs on a CUDA runtime thread: no CUDA calls here.
    auto *pr = static_cast<std::pair<fdtd_solver *, int> *>(arg);
    fdtd_solver *s = pr->first;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->filled.push_back(pr->second);
    }
    s->cv.notify_all();
    delete pr;
}

void writer_main(fdtd_solver *s)
{
    for (;;) {
        int slot;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait(lk, [&] { return s->stop || !s->filled.empty(); });
            if (s->filled.empty())
                return;
            slot = s->filled.front();
            s->filled.pop_front();
            s->writing++;
        }
        SnapshotSlot &sl = s->ring[slot];
        const size_t per = s->snap_floats_per_field;
        const int np = s->snap.nplanes;
        int st = FDTD_OK;
        if (s->snap.callback) {
            for (size_t k = 0; k < s->snap_fields.size(); k++)
                s->snap.callback(s->snap.user, sl.step, s->snap_fields[k], sl.host + k * per, s->snap.z0, np);
        } else {
            const int nf = (int)s->snap_fields.size();
            if (s->snap.format != FDTD_SNAPSHOT_BINARY) {
                std::vector<int> status(nf * np, FDTD_OK);
                parallel_for(nf * np, s->snap.writer_threads, [&](int j) {
                    const int k = j / np, z = j % np;
                    status[j] = write_plane_text(
                        snapshot_name(s->snap_dir.c_str(), s->snap_fields[k], sl.step, s->snap.z0 + z),
                        sl.host + k * per + (size_t)z * s->nx * s->ny, s->nx, s->ny);
                });
                for (int v : status)
                    if (v != FDTD_OK)
                        st = v;
            }
            if (s->snap.format != FDTD_SNAPSHOT_TEXT)
                for (int k = 0; k < nf; k++) {
                    const int v = write_floats(
                        snapshot_name_f32(s->snap_dir.c_str(), s->snap_fields[k], sl.step, s->snap.z0, np),
                        sl.host + k * per, per);
                    if (v != FDTD_OK)
                        st = v;
                }
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            sl.busy = false;
            s->writing--;
            if (st != FDTD_OK)
                s->writer_status = st;
        }
        s->cv.notify_all();
    }
}

int enqueue_snapshot(fdtd_solver *s, int step)
{
    // wait for a free ring slot (back-pressure on a slow consumer)
    SnapshotSlot *sl;
    int idx;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        idx = s->ring_next;
        sl = &s->ring[idx];
        s->cv.wait(lk, [&] { return !sl->busy; });
        sl->busy = true;
        sl->step = step;
        s->ring_next = (s->ring_next + 1) % (int)s->ring.size();
    }
    int st = FDTD_OK;
    if (s->copy_pending) {
        // The previous copy read buffers that the next step overwrites.
        st = cu(cudaStreamWaitEvent(s->stream, s->ev_copy, 0));
        s->copy_pending = false;
    }
    if (st == FDTD_OK)
        st = cu(cudaEventRecord(s->ev_step, s->stream));
    if (st == FDTD_OK)
        st = cu(cudaStreamWaitEvent(s->copy_stream, s->ev_step, 0));
    const size_t plane = (size_t)s->nx * s->ny;
    for (size_t k = 0; k < s->snap_fields.size() && st == FDTD_OK; k++) {
        const float *src = field_buffer(s, s->snap_fields[k], step + 1) + (size_t)s->snap.z0 * plane;
        st = cu(cudaMemcpyAsync(sl->host + k * s->snap_floats_per_field, src, sizeof(float) * s->snap_floats_per_field,
                                cudaMemcpyDeviceToHost, s->copy_stream));
    }
    if (st == FDTD_OK)
        st = cu(cudaEventRecord(s->ev_copy, s->copy_stream));
    if (st == FDTD_OK) {
        auto *arg = new std::pair<fdtd_solver *, int>(s, idx);
        st = cu(cudaLaunchHostFunc(s->copy_stream, snapshot_ready, arg));
        if (st != FDTD_OK)
            delete arg;
    }
    if (st != FDTD_OK) {
        std::lock_guard<std::mutex> lk(s->mu);
        sl->busy = false;
        return st;
    }
    s->copy_pending = true;
    s->copy_step = step;
    s->copy_gap = 2;
    if (s->kernel == FDTD_KERNEL_TWO_PASS)
        for (int f : s->snap_fields)
            if (f < 3)
                s->copy_gap = 1;
    return FDTD_OK;
}

void free_ring(fdtd_solver *s)
{
    for (auto &sl : s->ring)
        if (sl.host)
            cudaFreeHost(sl.host);
    s->ring.clear();
}

}  // namespace

extern "C" {

int fdtd_solver_create(const fdtd_solver_config *cfg, fdtd_solver **out)
{
    if (!cfg || !out || !cfg->params || !cfg->material || !cfg->specs)
        return FDTD_ERR_INVALID;
    if (cfg->kernel != FDTD_KERNEL_SINGLE_PASS && cfg->kernel != FDTD_KERNEL_TWO_PASS &&
        cfg->kernel != FDTD_KERNEL_COMPACT && cfg->kernel != FDTD_KERNEL_COMPACT_R16)
        return FDTD_ERR_INVALID;
    const FdtdParams *p = cfg->params;
    int st = cu(cudaSetDevice(cfg->device));
    if (st != FDTD_OK)
        return st;
    const size_t n = (size_t)p->nx * p->ny * p->nz;
    if (cfg->nclasses < 1 || cfg->nclasses > FDTD_MAX_CLASSES || plan_params_check(p, cfg->scheme) != FDTD_OK)
        return FDTD_ERR_INVALID;  // before any allocation
    auto *s = new (std::nothrow) fdtd_solver();
    if (!s)
        return FDTD_ERR_NOMEM;
    s->device = cfg->device;
    s->nx = p->nx; s->ny = p->ny; s->nz = p->nz;
    s->ncell = n;
    s->kernel = cfg->kernel;
    s->scheme = cfg->scheme;
    // The host scan of the class volume, then the plan, run on a helper
    // thread while this one allocates the state, has the device clear it and
    // uploads the volume.
    unsigned long long mhash = 0;
    int top = 0, helper_st = FDTD_OK;
    fdtd_plan *plan = nullptr;
    auto scan_and_plan = [&] {
        if (scan_material(cfg->material, p->nx, p->ny, p->nz, cfg->nclasses, &mhash, &top) != FDTD_OK) {
            helper_st = FDTD_ERR_INVALID;
            return;
        }
        helper_st = cu(cudaSetDevice(cfg->device));  // the current device is per thread
        if (helper_st == FDTD_OK)  // the classes up to the largest one present
            helper_st = fdtd_plan_create(p, cfg->specs, top + 1, cfg->scheme, nullptr, &plan);
    };
    std::thread helper;
    try {
        helper = std::thread(scan_and_plan);
    } catch (...) {
        scan_and_plan();  // no thread to be had: the same work in line
    }
    // H: two buffers for the single-pass kernels, one for the two-pass pair;
    // E: two slots; D: two slots, or one R array for the compact form (FP16
    // residuals and their scale words for the 16-bit form)
    const bool r16 = cfg->kernel == FDTD_KERNEL_COMPACT_R16;
    const int nh = cfg->kernel == FDTD_KERNEL_TWO_PASS ? 1 : 2;
    const int nd = stores_no_d(cfg->kernel) ? 1 : 2;
    const size_t fbytes = ((n * sizeof(float)) + 255) & ~size_t(255);
    const size_t dbytes = r16 ? ((n * sizeof(uint16_t)) + 255) & ~size_t(255) : fbytes;
    const size_t xbytes = r16 ? ((r16_words(p->nx, p->ny, p->nz) * sizeof(uint32_t)) + 255) & ~size_t(255) : 0;
    const size_t total = fbytes * (3 * nh + 6) + dbytes * 3 * nd + xbytes + ((n + 255) & ~size_t(255)) + 256;
    st = cu(cudaMalloc(&s->d_block, total));
    if (st == FDTD_OK) {
        char *q = s->d_block;
        for (int b = 0; b < nh; b++)
            for (int k = 0; k < 3; k++, q += fbytes)
                s->h[b][k] = reinterpret_cast<float *>(q);
        if (nh == 1)
            for (int k = 0; k < 3; k++)
                s->h[1][k] = s->h[0][k];
        for (int b = 0; b < 2; b++)
            for (int k = 0; k < 3; k++, q += fbytes)
                s->e[b][k] = reinterpret_cast<float *>(q);
        for (int b = 0; b < nd; b++)
            for (int k = 0; k < 3; k++, q += dbytes)
                s->d[b][k] = reinterpret_cast<float *>(q);
        if (nd == 1)
            for (int k = 0; k < 3; k++)
                s->d[1][k] = s->d[0][k];
        if (r16) {
            s->rexp = reinterpret_cast<uint32_t *>(q);
            q += xbytes;
        }
        s->mat = reinterpret_cast<uint8_t *>(q);
        q += (n + 255) & ~size_t(255);
        s->counter = reinterpret_cast<int *>(q);
        st = cu(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    }
    if (st == FDTD_OK)
        st = cu(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
    if (st == FDTD_OK)
        st = cu(cudaEventCreateWithFlags(&s->ev_step, cudaEventDisableTiming));
    if (st == FDTD_OK)
        st = cu(cudaEventCreateWithFlags(&s->ev_copy, cudaEventDisableTiming));
    if (st == FDTD_OK)
        st = cu(cudaMemsetAsync(s->d_block, 0, total, s->stream));
    if (st == FDTD_OK)
        st = cu(cudaMemcpyAsync(s->mat, cfg->material, n, cudaMemcpyHostToDevice, s->stream));
    if (helper.joinable())
        helper.join();
    s->plan = plan;  // destroyed with the solver on any failure below
    if (st == FDTD_OK)
        st = helper_st;
    // the classes up to the largest one present: the kernels stage that many
    // table entries
    const int ncls = top + 1;
    if (st == FDTD_OK) {
        s->nclasses = ncls;
        s->specs.assign(cfg->specs, cfg->specs + 4 * (size_t)ncls);
        s->material_hash = mhash;  // checkpoints must come from the same class volume
    }
    if (st == FDTD_OK && stores_no_d(cfg->kernel)) {
        // tile-planes without Debye memory: the strip kernel skips their R
        const std::vector<unsigned char> flags =
            strip_plane_flags(cfg->material, p->nx, p->ny, p->nz, p->nx, cfg->specs, ncls);
        s->memless_rows = strip_shape_rows(strip_single_shape(cfg->kernel == FDTD_KERNEL_COMPACT_R16));
        const int zchunk = strip_zchunk(p->nz);
        std::vector<unsigned long long> masks((size_t)((p->nz + zchunk - 1) / zchunk) *
                                              ((p->ny + s->memless_rows - 1) / s->memless_rows) * ((p->nx + 31) / 32));
        s->memless_fraction =
            strip_unit_masks(flags, p->nx, p->ny, p->nz, s->memless_rows, zchunk, masks.data());
        if (s->memless_fraction > 0.0) {
            st = cu(cudaMalloc(&s->d_memless, masks.size() * sizeof(unsigned long long)));
            if (st == FDTD_OK)
                st = cu(cudaMemcpyAsync(s->d_memless, masks.data(), masks.size() * sizeof(unsigned long long),
                                        cudaMemcpyHostToDevice, s->stream));
        }
    }
    if (st == FDTD_OK)
        st = cu(cudaStreamSynchronize(s->stream));
    if (st != FDTD_OK) {
        fdtd_solver_destroy(s);
        return st;
    }
    s->writer = std::thread(writer_main, s);
    *out = s;
    return FDTD_OK;
}

double fdtd_solver_memless_fraction(const fdtd_solver *s) { return s ? s->memless_fraction : 0.0; }

int fdtd_solver_destroy(fdtd_solver *s)
{
    if (!s)
        return FDTD_OK;
    cudaSetDevice(s->device);
    if (s->stream)
        cudaStreamSynchronize(s->stream);
    if (s->copy_stream)
        cudaStreamSynchronize(s->copy_stream);
    if (s->writer.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv.notify_all();
        s->writer.join();
    }
    reset_graphs(s);
    free_ring(s);
    if (s->d_probe_idx) cudaFree(s->d_probe_idx);
    if (s->d_probe_buf) cudaFree(s->d_probe_buf);
    if (s->d_dft) cudaFree(s->d_dft);
    if (s->ev_step) cudaEventDestroy(s->ev_step);
    if (s->ev_copy) cudaEventDestroy(s->ev_copy);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->d_block) cudaFree(s->d_block);
    if (s->d_memless) cudaFree(s->d_memless);
    fdtd_plan_destroy(s->plan);
    delete s;
    return FDTD_OK;
}

int fdtd_solver_run(fdtd_solver *s, int nsteps)
{
    if (!s || nsteps < 0)
        return FDTD_ERR_INVALID;
    int st = cu(cudaSetDevice(s->device));
    if (st != FDTD_OK)
        return st;
    if (s->snap.every <= 0)
        return launch_steps(s, nsteps);
    // run up to and including each snapshot step, then copy it out
    while (nsteps > 0) {
        const int every = s->snap.every;
        const int next_due = ((s->steps + every - 1) / every) * every;  // first step index >= steps with idx % every == 0
        const int len = std::min(nsteps, next_due - s->steps + 1);
        st = launch_steps(s, len);
        if (st != FDTD_OK)
            return st;
        nsteps -= len;
        if (s->steps - 1 == next_due) {
            st = enqueue_snapshot(s, next_due);
            if (st != FDTD_OK)
                return st;
        }
    }
    return FDTD_OK;
}

int fdtd_solver_synchronize(fdtd_solver *s)
{
    if (!s)
        return FDTD_ERR_INVALID;
    cudaSetDevice(s->device);
    int st = cu(cudaStreamSynchronize(s->stream));
    if (st == FDTD_OK)
        st = plan_error(s->plan);
    return st;
}

int fdtd_solver_steps(const fdtd_solver *s) { return s ? s->steps : -1; }

int fdtd_solver_test_stall(fdtd_solver *s)
{
    if (!s)
        return FDTD_ERR_INVALID;
    cudaSetDevice(s->device);
    static const int one = 1;
    int st = cu(cudaMemcpyAsync(s->plan->d_stall, &one, sizeof one, cudaMemcpyHostToDevice, s->stream));
    if (st == FDTD_OK)
        st = cu(cudaStreamSynchronize(s->stream));  // the source is host memory of this call
    return st;
}

fdtd_stream_t fdtd_solver_stream(const fdtd_solver *s) { return s ? s->stream : nullptr; }

int fdtd_solver_get_field(fdtd_solver *s, int field, float *host_out)
{
    if (!s || !host_out || field < 0 || field >= FDTD_FIELD_COUNT)
        return FDTD_ERR_INVALID;
    const float *src = field_buffer(s, field, s->steps);
    if (!src)
        return FDTD_ERR_INVALID;
    int st = fdtd_solver_synchronize(s);
    if (st == FDTD_OK)
        st = cu(cudaMemcpy(host_out, src, sizeof(float) * s->ncell, cudaMemcpyDeviceToHost));
    return st;
}

int fdtd_solver_set_snapshots(fdtd_solver *s, const fdtd_snapshot_spec *spec)
{
    if (!s || !spec)
        return FDTD_ERR_INVALID;
    int st = fdtd_solver_flush_snapshots(s);
    if (st != FDTD_OK)
        return st;
    free_ring(s);
    s->snap = fdtd_snapshot_spec{};
    s->snap_fields.clear();
    if (spec->every <= 0)
        return FDTD_OK;
    fdtd_snapshot_spec sp = *spec;
    if (sp.nplanes == 0) {
        sp.z0 = 0;
        sp.nplanes = s->nz;
    }
    if (sp.z0 < 0 || sp.nplanes < 0 || sp.z0 + sp.nplanes > s->nz || (sp.field_mask & ((1u << FDTD_FIELD_COUNT) - 1)) == 0)
        return FDTD_ERR_INVALID;
    if (!sp.callback && !sp.output_dir)
        return FDTD_ERR_INVALID;
    if (sp.format < FDTD_SNAPSHOT_TEXT || sp.format > FDTD_SNAPSHOT_TEXT_AND_BINARY)
        return FDTD_ERR_INVALID;
    if (stores_no_d(s->kernel) && (sp.field_mask & (7u << FDTD_FIELD_DX)))
        return FDTD_ERR_INVALID;  // D is not stored
    for (int f = 0; f < FDTD_FIELD_COUNT; f++)
        if (sp.field_mask & (1u << f))
            s->snap_fields.push_back(f);
    s->snap_dir = sp.output_dir ? sp.output_dir : "";
    sp.output_dir = nullptr;
    s->snap_floats_per_field = (size_t)s->nx * s->ny * sp.nplanes;
    const size_t bytes = sizeof(float) * s->snap_floats_per_field * s->snap_fields.size();
    const int nslots = bytes > (size_t(1) << 30) ? 2 : 3;
    s->ring.resize(nslots);
    for (auto &sl : s->ring) {
        st = cu(cudaHostAlloc(&sl.host, bytes, cudaHostAllocDefault));
        if (st != FDTD_OK) {
            free_ring(s);
            s->snap_fields.clear();
            return st;
        }
    }
    s->ring_next = 0;
    s->snap = sp;
    return FDTD_OK;
}

int fdtd_solver_profile(fdtd_solver *s, int nsteps, float *avg_ms, int max_kernels, int *nkernels)
{
    if (!s || nsteps < 1 || !avg_ms || max_kernels < 1 || !nkernels)
        return FDTD_ERR_INVALID;
    int st = cu(cudaSetDevice(s->device));
    if (st != FDTD_OK)
        return st;
    if (s->copy_pending) {
        st = cu(cudaStreamWaitEvent(s->stream, s->ev_copy, 0));
        s->copy_pending = false;
    }
    StepKernel ks[8];
    const int nk = step_kernels(s->kernel, solver_consts(s, s->steps), ks, 8);
    std::vector<cudaEvent_t> ev((size_t)nsteps * (nk + 1), nullptr);
    for (auto &e : ev)
        if (st == FDTD_OK)
            st = cu(cudaEventCreate(&e));
    for (int k = 0; k < nsteps && st == FDTD_OK; k++) {
        const int n = s->steps;
        NativeConsts c = solver_consts(s, n);
        c.step_counter = s->counter;
        c.fuse_mur_x = s->kernel != FDTD_KERNEL_TWO_PASS;  // as launch_step sets it
        cudaEvent_t *e = &ev[(size_t)k * (nk + 1)];
        st = cu(cudaEventRecord(e[0], s->stream));
        for (int j = 0; j < nk && st == FDTD_OK; j++) {
            st = ks[j].launch(c, s->stream);
            if (st == FDTD_OK)
                st = cu(cudaEventRecord(e[j + 1], s->stream));
        }
        s->steps++;
    }
    if (st == FDTD_OK)
        st = cu(cudaStreamSynchronize(s->stream));
    std::vector<double> sum(nk, 0.0);
    for (int k = 0; k < nsteps && st == FDTD_OK; k++)
        for (int j = 0; j < nk && st == FDTD_OK; j++) {
            float ms = 0.0f;
            st = cu(cudaEventElapsedTime(&ms, ev[(size_t)k * (nk + 1) + j], ev[(size_t)k * (nk + 1) + j + 1]));
            sum[j] += ms;
        }
    for (auto &e : ev)
        if (e)
            cudaEventDestroy(e);
    if (st != FDTD_OK)
        return st;
    for (int j = 0; j < nk && j < max_kernels; j++)
        avg_ms[j] = (float)(sum[j] / nsteps);
    *nkernels = nk;
    return FDTD_OK;
}

const char *fdtd_solver_kernel_name(const fdtd_solver *s, int k)
{
    if (!s || k < 0)
        return nullptr;
    StepKernel ks[8];
    const int nk = step_kernels(s->kernel, solver_consts(s, s->steps), ks, 8);
    return k < nk ? ks[k].name : nullptr;
}

int fdtd_solver_flush_snapshots(fdtd_solver *s)
{
    if (!s)
        return FDTD_ERR_INVALID;
    cudaSetDevice(s->device);
    int st = cu(cudaStreamSynchronize(s->copy_stream));
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv.wait(lk, [&] { return s->filled.empty() && s->writing == 0; });
    if (st == FDTD_OK && s->writer_status != FDTD_OK) {
        st = s->writer_status;
        s->writer_status = FDTD_OK;
    }
    return st;
}

}  // extern "C"
