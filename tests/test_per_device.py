"""Per-device one-time set-up (fdtd_gb300/csrc/per_device.h), on the CPU.

The kernels' dynamic shared-memory opt-in (cudaFuncSetAttribute) holds for
the current device only, so the launchers make it once per device through
PerDeviceOnce.  This test compiles the header into a small host program and
checks the bookkeeping with fake device indices: one set-up per device, a
failed set-up retried, out-of-range devices refused, concurrent first calls
running the set-up once."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

PROGRAM = r"""
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>
#include "per_device.h"

int main()
{
    fdtd::PerDeviceOnce<4> once;
    int calls[4] = {0, 0, 0, 0};
    auto setup = [&](int dev, int status) { return [&, dev, status] { calls[dev]++; return status; }; };
    if (once.run(0, setup(0, 0)) != 0 || once.run(0, setup(0, 0)) != 0 || calls[0] != 1) return 1;
    if (once.done(1) || once.run(1, setup(1, 0)) != 0 || calls[1] != 1 || !once.done(1)) return 2;
    if (once.run(2, setup(2, 7)) != 7 || once.done(2)) return 3;          // failure reported, not recorded
    if (once.run(2, setup(2, 0)) != 0 || calls[2] != 2 || !once.done(2)) return 4;  // retried
    if (once.run(4, setup(3, 0)) != -1 || once.run(-1, setup(3, 0)) != -1 || calls[3] != 0) return 5;
    fdtd::PerDeviceOnce<4> shared;
    std::atomic<int> n{0};
    std::vector<std::thread> ts;
    for (int t = 0; t < 8; t++)
        ts.emplace_back([&] { shared.run(3, [&] { n++; return 0; }); });
    for (auto &t : ts) t.join();
    if (n != 1) return 6;
    std::puts("ok");
    return 0;
}
"""


def test_per_device_once(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = tmp_path / "t.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "t"
    subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", f"-I{ROOT / 'fdtd_gb300' / 'csrc'}", str(src), "-o",
                    str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", (out.returncode, out.stdout, out.stderr)
