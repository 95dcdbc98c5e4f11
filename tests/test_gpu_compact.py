"""Compact nine-field form (FDTD_KERNEL_COMPACT): the same Debye update as
updateEField (fdtd_calculations.cu:141-183) with D and E^{n-1} folded into one
recursion variable R per component.  Its fields must agree with the oracle and
the D-form kernel within the FP32 tolerance; D is not stored."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from fdtd_gb300 import phantom as ph
from oracle import pyoracle as po

from .gpu_util import Params, make_params
from .helpers import REL_L2_TOL, assert_fields_close, class_media, random_case, rel_l2

pytestmark = pytest.mark.gpu

EH = ("hx", "hy", "hz", "ex", "ey", "ez")


def _sphere(root, n, t_max, kernel, scheme, timeskip=None):
    path = ph.c1_inputs(root, n=n, t_max=t_max)
    p = fg.Params.read(path)
    if timeskip is not None:
        p.set_timeskip(timeskip)
    codes = fg.load_material_codes(p, root / "pgm")
    specs = fg.read_specs(root / "mat_specs")
    return p, codes, specs, fg.Solver(p, codes, specs, scheme=scheme, kernel=kernel, nclasses=2)


def _oracle_sphere(root, p, codes, specs, steps, corrected):
    q = po.params_read(root / "input_params", "f64" if corrected else "f32")
    q.dt = p.dt
    jz = p.setup_sources()
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    media.rp = po.uniform_media(q).rp
    n = p.nx
    st = po.State(n, p.ny, p.nz, np.float64 if corrected else np.float32)
    po.run(po.make_cfg(q, jz, corrected=corrected), media, st, 0, steps)
    return st.latest(steps)


def test_compact_corrected_scheme_vs_fp64_oracle(cuda, tmp_path):
    """64^3 sphere, dt = 0.99 of the Courant limit, 501 steps."""
    p, codes, specs, s = _sphere(tmp_path, 64, 500, fg.KERNEL_COMPACT, fg.SCHEME_CORRECTED, timeskip=0.99)
    steps = p.iterationsCount
    s.run(steps)
    got = s.fields()
    s.close()
    assert sorted(got) == sorted(EH)
    want = _oracle_sphere(tmp_path, p, codes, specs, steps, corrected=True)
    assert max(np.abs(want[k]).max() for k in EH) > 0
    assert_fields_close(got, want, tol=REL_L2_TOL, names=EH)


def test_compact_reference_scheme_finite_window(cuda, tmp_path):
    """Reference scheme, 60 steps (the fields stay finite): against the FP32
    oracle that reproduces the reference kernels."""
    p, codes, specs, s = _sphere(tmp_path, 64, 60, fg.KERNEL_COMPACT, fg.SCHEME_REFERENCE)
    s.run(60)
    got = s.fields()
    s.close()
    want = _oracle_sphere(tmp_path, p, codes, specs, 60, corrected=False)
    assert all(np.all(np.isfinite(want[k])) for k in EH)
    assert_fields_close(got, want, names=EH)


@pytest.mark.parametrize("dims", [(48, 40, 36), (37, 29, 23)])  # TMA path; cp.async path (nx % 4 != 0)
def test_compact_dispersive_media_vs_oracle_and_d_form(cuda, dims):
    """Random Debye classes (strong dispersion), two sources, random Mur
    slabs: compact form against the FP64 oracle and the D-form kernel."""
    steps = 80
    codes, specs, rp, sources, consts, jz = random_case(*dims, seed=7, ncls=5, nsrc=2)
    raw = make_params(dims, consts, sources, jz)
    with fg.Solver(Params(raw), codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=fg.KERNEL_COMPACT) as s:
        s.run(33)
        s.run(steps - 33)
        got = s.fields()
    with fg.Solver(Params(raw), codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=fg.KERNEL_SINGLE_PASS) as s:
        s.run(steps)
        dform = s.fields()
    p = po.OracleParams()
    p.nx, p.ny, p.nz = dims
    p.pi, p.wave_frequency, p.eps0 = raw.pi, raw.waveFrequency, raw.eps0
    p.default_sigma, p.default_eps_s = raw.defaultSigma, raw.defaultEpsS
    p.default_eps_i, p.default_tau_d = raw.defaultEpsI, raw.defaultTauD
    media = class_media(codes, specs, po.uniform_media(p).rp)
    st = po.State(*dims, np.float64)
    po.run(po.make_cfg(dims, jz, sources=sources, consts=consts, corrected=True), media, st, 0, steps)
    want = st.latest(steps)
    assert_fields_close(got, want, names=EH)
    # both FP32 forms are within the tolerance of the FP64 solution, so they
    # are within twice of it from each other
    assert_fields_close(got, dform, tol=2 * REL_L2_TOL, names=EH)


def test_compact_has_no_d_fields(cuda, tmp_path):
    p, codes, specs, s = _sphere(tmp_path, 16, 9, fg.KERNEL_COMPACT, fg.SCHEME_CORRECTED)
    s.run(2)
    with pytest.raises(fg.FdtdError) as e:
        s.field("dz")
    assert e.value.status == fg.FDTD_ERR_INVALID
    with pytest.raises(fg.FdtdError):
        s.set_snapshots(every=1, fields=("ez", "dz"), callback=lambda *a: None)
    s.set_snapshots(every=1, fields=("ez",), callback=lambda *a: None)
    s.run(2)
    s.flush_snapshots()
    assert set(s.profile(2)) == {"compact_step", "mur"}
    s.close()


@pytest.mark.parametrize("at", [0, 11])
def test_compact_checkpoint_resume_is_bit_identical(cuda, tmp_path, at):
    p, codes, specs, a = _sphere(tmp_path / "a", 32, 60, fg.KERNEL_COMPACT, fg.SCHEME_CORRECTED, timeskip=0.99)
    a.run(at)
    a.checkpoint(tmp_path / "ck.bin")
    a.run(40 - at)
    want = a.fields()
    a.close()
    _, _, _, b = _sphere(tmp_path / "b", 32, 60, fg.KERNEL_COMPACT, fg.SCHEME_CORRECTED, timeskip=0.99)
    b.run(5)
    b.restore(tmp_path / "ck.bin")
    assert b.steps == at
    b.run(40 - at)
    got = b.fields()
    b.close()
    for k in want:
        assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), k
    # a D-form solver does not take a compact checkpoint
    _, _, _, c = _sphere(tmp_path / "c", 32, 60, fg.KERNEL_SINGLE_PASS, fg.SCHEME_CORRECTED, timeskip=0.99)
    with pytest.raises(fg.FdtdError) as e:
        c.restore(tmp_path / "ck.bin")
    assert e.value.status == fg.FDTD_ERR_FORMAT
    c.close()


def test_compact_probes_match_d_form(cuda, tmp_path):
    """On-device probes and DFT read E only, so they work on the compact form."""
    out = {}
    for kernel in (fg.KERNEL_SINGLE_PASS, fg.KERNEL_COMPACT):
        p, codes, specs, s = _sphere(tmp_path / str(kernel), 24, 90, kernel, fg.SCHEME_CORRECTED, timeskip=0.99)
        s.set_probes([(12, 12, 12), (4, 6, 8)], capacity=90)
        s.set_dft(1.0e9, stride=3)
        s.run(90)
        out[kernel] = (s.probes(), s.dft(2))
        s.close()
    a, b = out[fg.KERNEL_SINGLE_PASS], out[fg.KERNEL_COMPACT]
    assert rel_l2(b[0], a[0]) < REL_L2_TOL
    assert np.linalg.norm(b[1] - a[1]) / np.linalg.norm(a[1]) < REL_L2_TOL
