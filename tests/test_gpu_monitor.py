"""Checkpoint/resume and the on-device monitors (probes, DFT, SAR) of the
solver, against uninterrupted runs and the FP64 oracle."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from fdtd_gb300 import phantom as ph
from oracle import pyoracle as po

from .helpers import rel_l2

pytestmark = pytest.mark.gpu


def _solver(root, n, kernel=fg.KERNEL_SINGLE_PASS, scheme=fg.SCHEME_CORRECTED):
    path = ph.c1_inputs(root, n=n, t_max=300)
    p = fg.Params.read(path)
    p.set_timeskip(0.99)
    codes = fg.load_material_codes(p, root / "pgm")
    specs = fg.read_specs(root / "mat_specs")
    return p, codes, specs, fg.Solver(p, codes, specs, scheme=scheme, kernel=kernel, nclasses=2)


@pytest.mark.parametrize("kernel", [fg.KERNEL_SINGLE_PASS, fg.KERNEL_TWO_PASS])
@pytest.mark.parametrize("at", [0, 7, 30])
def test_checkpoint_resume_is_bit_identical(cuda, tmp_path, kernel, at):
    p, codes, specs, a = _solver(tmp_path / "a", 32, kernel)
    a.run(at)
    a.checkpoint(tmp_path / "ck.bin")
    a.run(45 - at)
    want = a.fields()
    a.close()
    _, _, _, b = _solver(tmp_path / "b", 32, kernel)
    b.run(3)  # state to be overwritten
    b.restore(tmp_path / "ck.bin")
    assert b.steps == at
    b.run(45 - at)
    got = b.fields()
    b.close()
    for k in want:
        assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), k


def test_restore_rejects_other_configuration(cuda, tmp_path):
    p, codes, specs, a = _solver(tmp_path / "a", 24)
    a.run(2)
    a.checkpoint(tmp_path / "ck.bin")
    a.close()
    _, _, _, b = _solver(tmp_path / "b", 24, scheme=fg.SCHEME_REFERENCE)
    with pytest.raises(fg.FdtdError) as e:
        b.restore(tmp_path / "ck.bin")
    assert e.value.status == fg.FDTD_ERR_FORMAT
    b.close()


def test_probes_dft_and_sar_against_fp64_oracle(cuda, tmp_path):
    n, steps, stride, freq = 32, 240, 4, 1.0e9
    p, codes, specs, s = _solver(tmp_path, n)
    probes = [(20, 16, 16), (16, 16, 16), (5, 9, 20)]
    s.set_probes(probes, capacity=steps)
    s.set_dft(freq, stride=stride, z0=10, nplanes=12)
    s.run(steps)
    series = s.probes()
    acc = [s.dft(c) for c in range(3)]
    peak, cell = s.peak_sar()
    s.close()
    assert series.shape == (steps, 3, 3)

    # FP64 oracle, same steps, same accumulation rule
    q = po.params_read(tmp_path / "input_params", "f64")
    q.dt = p.dt
    jz = p.setup_sources()
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    media.rp = po.uniform_media(q).rp
    cfg = po.make_cfg(q, jz, corrected=True)
    st = po.State(n, n, n, np.float64)
    want_series = np.zeros((steps, 3, 3))
    want_acc = [np.zeros((12, n, n), complex) for _ in range(3)]
    for k in range(steps):
        po.run(cfg, media, st, k, 1)
        e = st.e[k % 3]
        for j, (x, y, z) in enumerate(probes):
            want_series[k, j] = [e[c][z, y, x] for c in range(3)]
        m = k + 1
        if m % stride == 0:
            ph_ = np.exp(-1j * 2 * np.pi * freq * m * float(p.dt)) * stride * float(p.dt)
            for c in range(3):
                want_acc[c] += e[c][10:22] * ph_
    assert rel_l2(series, want_series) < 1e-5
    for c in range(3):
        num = np.linalg.norm(acc[c] - want_acc[c])
        assert num / np.linalg.norm(want_acc[c]) < 1e-5
    sig = specs[codes[10:22], 0].astype(np.float64)
    sar = sig * sum(np.abs(a) ** 2 for a in want_acc) / (2 * 1000.0)
    assert abs(peak - sar.max()) / sar.max() < 1e-5
    assert cell == 10 * n * n + int(np.argmax(sar))
