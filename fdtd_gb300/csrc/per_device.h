// per_device.h -- one-time set-up per CUDA device.
//
// Some CUDA settings apply to the current device only; the dynamic
// shared-memory opt-in that cudaFuncSetAttribute records for a kernel is one
// of them.  A process-wide std::call_once would configure the first device
// and leave every other device to fail its launches, so each such setting is
// made once per device instead, on the first use on that device.  Host code
// only; no CUDA types, so the bookkeeping compiles and is tested without a
// GPU.
#pragma once

#include <mutex>

namespace fdtd {

template <int MAX_DEVICES = 64>
class PerDeviceOnce {
public:
    // Runs setup() for device dev unless it already succeeded there.  setup
    // returns 0 on success; a failed set-up is retried on the next call.
    // Returns setup's status, 0 when there was nothing to do, or -1 for a
    // device index outside [0, MAX_DEVICES).
    template <class F>
    int run(int dev, F &&setup)
    {
        if (dev < 0 || dev >= MAX_DEVICES)
            return -1;
        std::lock_guard<std::mutex> lock(mu_);
        if (done_[dev])
            return 0;
        const int st = setup();
        if (st == 0)
            done_[dev] = true;
        return st;
    }

    bool done(int dev) const { return dev >= 0 && dev < MAX_DEVICES && done_[dev]; }

private:
    std::mutex mu_;
    bool done_[MAX_DEVICES] = {};
};

}  // namespace fdtd
