// solver_internal.cuh -- the solver object shared by solver.cu and monitor.cu.
#pragma once

#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "native.cuh"

namespace fdtd {

struct SnapshotSlot {
    float *host = nullptr;  // pinned
    int step = -1;
    bool busy = false;      // filled or being filled
};

}  // namespace fdtd

struct fdtd_solver {
    int device = 0;
    int nx = 0, ny = 0, nz = 0;
    size_t ncell = 0;
    int kernel = FDTD_KERNEL_SINGLE_PASS;
    fdtd_plan *plan = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;
    char *d_block = nullptr;
    float *h[2][3] = {};
    float *e[2][3] = {};
    float *d[2][3] = {};
    uint8_t *mat = nullptr;
    uint32_t *rexp = nullptr;  // FDTD_KERNEL_COMPACT_R16: scale words (d[0] holds the FP16 residuals)
    unsigned long long *d_memless = nullptr;  // compact forms: the strip kernel's memoryless-plane masks
    double memless_fraction = 0.0;            // share of the cell-updates on such planes
    int memless_rows = 0;                     // tile rows of those masks
    int *counter = nullptr;
    int steps = 0;
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (parity, length) -> exec
    // snapshots
    fdtd_snapshot_spec snap{};
    std::string snap_dir;
    std::vector<int> snap_fields;
    size_t snap_floats_per_field = 0;
    std::vector<fdtd::SnapshotSlot> ring;
    int ring_next = 0;
    cudaEvent_t ev_step = nullptr, ev_copy = nullptr;
    bool copy_pending = false;  // a snapshot copy must finish before step copy_step + copy_gap
    int copy_step = -1;
    int copy_gap = 2;           // 1 when H is copied and updated in place
    std::mutex mu;
    std::condition_variable cv;
    std::deque<int> filled;     // ring slot indices ready for the writer
    int writing = 0;
    bool stop = false;
    int writer_status = FDTD_OK;
    std::thread writer;
    // configuration kept for checkpoints and SAR
    int scheme = FDTD_SCHEME_REFERENCE;
    int nclasses = 0;
    unsigned long long material_hash = 0;
    std::vector<float> specs;  // nclasses x 4
    // probes
    int nprobes = 0, probe_cap = 0, probe_start = 0;
    long long *d_probe_idx = nullptr;
    float *d_probe_buf = nullptr;
    // running DFT
    bool dft_on = false;
    double dft_freq = 0.0;
    int dft_stride = 1, dft_z0 = 0, dft_np = 0;
    double *d_dft = nullptr;  // re x,y,z then im x,y,z, nx*ny*dft_np each
};

namespace fdtd {

// Pointers of step n and the device buffer of a field after `count` steps.
fdtd_native_fields step_fields(const fdtd_solver *s, int n);
// Kernel arguments of step n (the form's extra state included).
NativeConsts solver_consts(const fdtd_solver *s, int n);
// The form stores no D (the compact forms).
inline bool stores_no_d(int kernel) { return kernel == FDTD_KERNEL_COMPACT || kernel == FDTD_KERNEL_COMPACT_R16; }
const float *field_buffer(const fdtd_solver *s, int field, int count);
// Monitor launch after step n (nothing when no monitor is installed).
int launch_monitor(fdtd_solver *s, int n);
// Drops the captured step graphs (the monitor set changed).
void reset_graphs(fdtd_solver *s);

}  // namespace fdtd

