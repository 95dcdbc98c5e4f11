"""Compact form with R stored in 16 bits (FDTD_KERNEL_COMPACT_R16): the
compact form's update (updateEField, fdtd_calculations.cu:141-183, with D and
E^{n-1} folded into R) with the residual R^{n+1} + a E^{n+1} held as an FP16
value per cell and one power-of-two scale per 32-cell
row segment.  H, E and the arithmetic stay FP32, so the form is judged
against the FP64 oracle at the reduced-storage tolerance R16_TOL (relative L2
of each field and of each probe's E series), and against the 32-bit compact
form."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from fdtd_gb300 import phantom as ph
from oracle import pyoracle as po

from .gpu_util import Params, make_params
from .helpers import REL_L2_TOL, class_media, random_case, rel_l2

pytestmark = pytest.mark.gpu

EH = ("hx", "hy", "hz", "ex", "ey", "ez")
R16_TOL = 1e-3  # relative L2 against the FP64 oracle: every E and H field, every probe's E series


def _sphere(root, n, t_max, kernel, timeskip=0.99):
    path = ph.c1_inputs(root, n=n, t_max=t_max)
    p = fg.Params.read(path)
    p.set_timeskip(timeskip)
    codes = fg.load_material_codes(p, root / "pgm")
    specs = fg.read_specs(root / "mat_specs")
    return p, codes, specs, fg.Solver(p, codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel, nclasses=2)


def test_compact16_sphere_fields_and_probes_vs_fp64_oracle(cuda, tmp_path):
    """64^3 Debye sphere, dt = 0.99 of the Courant limit, 501 steps: E and H
    and the E series at probes inside and outside the sphere, among them
    cells on the source's row (y = z = 32), where the dipole's near field
    makes one 32-cell segment span more than three decades: FP16 keeps 11
    significant bits for every value of a segment, so the small ones there
    lose nothing to the segment's scale."""
    p, codes, specs, s = _sphere(tmp_path, 64, 500, fg.KERNEL_COMPACT_R16)
    steps = p.iterationsCount
    probes = [(32, 32, 32), (20, 32, 32), (31, 32, 32), (40, 30, 28), (24, 36, 34), (50, 50, 50), (32, 40, 32),
              (45, 20, 44)]
    s.set_probes(probes, capacity=steps)
    s.run(steps)
    got = s.fields()
    series = s.probes().astype(np.float64)
    assert set(s.profile(2)) == {"compact16_step", "mur"}
    s.close()
    assert sorted(got) == sorted(EH)

    q = po.params_read(tmp_path / "input_params", "f64")
    q.dt = p.dt
    jz = p.setup_sources()
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    media.rp = po.uniform_media(q).rp
    cfg = po.make_cfg(q, jz, corrected=True)
    st = po.State(64, 64, 64, np.float64)
    want_series = np.zeros((steps, len(probes), 3))
    for k in range(steps):
        po.run(cfg, media, st, k, 1)
        e = st.e[k % 3]
        for j, (x, y, z) in enumerate(probes):
            want_series[k, j] = [e[c][z, y, x] for c in range(3)]
    want = st.latest(steps)
    errs = {n: rel_l2(got[n], want[n]) for n in EH}
    assert max(errs.values()) <= R16_TOL, errs
    per_probe = [rel_l2(series[:, j], want_series[:, j]) for j in range(len(probes))]
    assert max(per_probe) <= R16_TOL, per_probe
    # the 16-bit storage is visible: not the 32-bit compact form's bits
    assert max(errs.values()) > REL_L2_TOL / 100


@pytest.mark.parametrize("dims", [(48, 40, 36), (37, 29, 23), (33, 7, 5), (64, 17, 65)])  # TMA / direct-load paths
def test_compact16_dispersive_media_vs_oracle_and_compact(cuda, dims):
    """Random Debye classes, two sources, random Mur slabs; grids whose rows
    are staged by TMA (nx % 16 == 0) and grids whose R is read directly."""
    steps = 80
    codes, specs, rp, sources, consts, jz = random_case(*dims, seed=11, ncls=5, nsrc=2)
    raw = make_params(dims, consts, sources, jz)
    with fg.Solver(Params(raw), codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=fg.KERNEL_COMPACT_R16) as s:
        s.run(29)
        s.run(steps - 29)
        got = s.fields()
    with fg.Solver(Params(raw), codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=fg.KERNEL_COMPACT) as s:
        s.run(steps)
        compact = s.fields()
    p = po.OracleParams()
    p.nx, p.ny, p.nz = dims
    p.pi, p.wave_frequency, p.eps0 = raw.pi, raw.waveFrequency, raw.eps0
    p.default_sigma, p.default_eps_s = raw.defaultSigma, raw.defaultEpsS
    p.default_eps_i, p.default_tau_d = raw.defaultEpsI, raw.defaultTauD
    media = class_media(codes, specs, po.uniform_media(p).rp)
    st = po.State(*dims, np.float64)
    po.run(po.make_cfg(dims, jz, sources=sources, consts=consts, corrected=True), media, st, 0, steps)
    want = st.latest(steps)
    for n in EH:
        assert np.all(np.isfinite(got[n])), n
        assert rel_l2(got[n], want[n]) <= R16_TOL, (n, rel_l2(got[n], want[n]))
        assert rel_l2(got[n], compact[n]) <= R16_TOL, (n, rel_l2(got[n], compact[n]))


def test_compact16_has_no_d_fields_and_zero_steps_stay_zero(cuda, tmp_path):
    p, codes, specs, s = _sphere(tmp_path, 16, 9, fg.KERNEL_COMPACT_R16)
    assert all(not np.any(v) for v in s.fields().values())
    s.run(2)
    with pytest.raises(fg.FdtdError) as e:
        s.field("dz")
    assert e.value.status == fg.FDTD_ERR_INVALID
    with pytest.raises(fg.FdtdError):
        s.set_snapshots(every=1, fields=("ez", "dz"), callback=lambda *a: None)
    s.close()


@pytest.mark.parametrize("at", [0, 13])
def test_compact16_checkpoint_resume_is_bit_identical(cuda, tmp_path, at):
    """The checkpoint holds the FP16 residuals and their scale words as stored."""
    p, codes, specs, a = _sphere(tmp_path / "a", 32, 60, fg.KERNEL_COMPACT_R16)
    a.run(at)
    a.checkpoint(tmp_path / "ck.bin")
    a.run(40 - at)
    want = a.fields()
    a.close()
    _, _, _, b = _sphere(tmp_path / "b", 32, 60, fg.KERNEL_COMPACT_R16)
    b.run(5)
    b.restore(tmp_path / "ck.bin")
    assert b.steps == at
    b.run(40 - at)
    got = b.fields()
    b.close()
    for k in want:
        assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), k
    # the 32-bit compact form does not take this checkpoint
    _, _, _, c = _sphere(tmp_path / "c", 32, 60, fg.KERNEL_COMPACT)
    with pytest.raises(fg.FdtdError) as e:
        c.restore(tmp_path / "ck.bin")
    assert e.value.status == fg.FDTD_ERR_FORMAT
    c.close()
