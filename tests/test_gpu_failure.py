"""Failure path of the single-pass kernels on the GPU, without a GPU fault.

A test hook (fdtd_solver_test_stall) makes the first CTA of the next step arm
one plane's mbarrier without issuing the copies, so that CTA's bounded wait
(0.2 s of the global timer) runs out.  The CTA raises the solver's error flag
and exits; the launch completes.  The solver must report
FDTD_ERR_DEVICE_TIMEOUT once, soon, and the device context must stay usable:
a checkpoint taken before the failed step, restored, must give the fields of
an undisturbed run bit for bit."""
from __future__ import annotations

import time

import numpy as np
import pytest

import fdtd_gb300 as fg
from fdtd_gb300 import phantom as ph

pytestmark = pytest.mark.gpu


def _solver(root, kernel):
    path = ph.c1_inputs(root, n=32, t_max=60)  # nx = 32: TMA staging
    p = fg.Params.read(path)
    p.set_timeskip(0.99)
    codes = fg.load_material_codes(p, root / "pgm")
    specs = fg.read_specs(root / "mat_specs")
    return fg.Solver(p, codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel, nclasses=2)


@pytest.mark.parametrize("kernel", [fg.KERNEL_SINGLE_PASS, fg.KERNEL_COMPACT])
def test_timed_out_wait_is_reported_and_the_context_survives(cuda, tmp_path, kernel):
    with _solver(tmp_path / "a", kernel) as s:
        s.run(10)
        s.checkpoint(tmp_path / "ck.bin")
        s.test_stall()
        t0 = time.perf_counter()
        s.run(1)
        with pytest.raises(fg.FdtdError) as e:
            s.synchronize()
        elapsed = time.perf_counter() - t0
        assert e.value.status == fg.FDTD_ERR_DEVICE_TIMEOUT
        assert elapsed < 5.0, elapsed
        s.synchronize()  # reported once; the flag is clear again
        s.run(3)         # later steps run normally (their fields are not checked:
        s.synchronize()  # the failed step left one tile behind)
        s.restore(tmp_path / "ck.bin")
        assert s.steps == 10
        s.run(20)
        got = s.fields()
    with _solver(tmp_path / "b", kernel) as s:
        s.run(30)
        want = s.fields()
    for name in want:
        assert np.array_equal(got[name].view(np.uint32), want[name].view(np.uint32)), name
