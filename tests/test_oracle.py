"""The oracle is pinned against fixtures produced by the reference itself."""
from __future__ import annotations

import json

import numpy as np
import pytest

from oracle import build as obuild
from oracle import pyoracle as po

from .helpers import RUNS, bits_equal, load_run, random_case, class_media, rel_l2


@pytest.mark.parametrize("name", RUNS)
def test_fp32_oracle_reproduces_reference_run_bit_for_bit(name):
    g = load_run(name)
    st = po.State(*g.dims, np.float32)
    po.run(g.cfg(), g.media, st, 0, g.steps)
    for k, (got, want) in enumerate(zip(st.arrays(), g.state)):
        assert bits_equal(got, want), f"array {k} differs"


@pytest.mark.parametrize("name", RUNS)
def test_fp64_oracle_close_to_reference_run(name):
    g = load_run(name)
    st = po.State(*g.dims, np.float64)
    po.run(g.cfg(), g.media, st, 0, g.steps)
    for k, (got, want) in enumerate(zip(st.arrays(), g.state)):
        assert rel_l2(want, got) < 1e-5, f"array {k}"


def test_oracle_params_and_source_table_match_reference(golden, tmp_path):
    for case in ("vacuum3ghz", "sphere1ghz", "debye900"):
        rec = json.loads((golden / f"params_{case}.json").read_text())
        path = tmp_path / f"input_params_{case}"
        path.write_text(rec["input_params"])
        p = po.params_read(path, "f64")
        for k, bits in rec["params_f32_hex"].items():
            assert np.float32(getattr(p, k)).view(np.uint32) == bits, (case, k)
        for k, v in rec["params"].items():
            if not isinstance(v, float):
                assert getattr(p, k) == v, (case, k)
        assert [list(s) for s in p.source_list()] == rec["sources"]
        jz = po.setup_sources(p, "f64")
        want = np.load(golden / f"jz_{case}.npy")
        assert bits_equal(jz[: want.size], want)
        assert not np.any(jz[want.size:1 << 14])


def test_oracle_materials_match_reference(golden, tmp_path):
    z = np.load(golden / "materials.npz")
    nx, ny, nz = (int(v) for v in z["dims"])
    (tmp_path / "mat_specs").write_text(str(z["specs_text"]))
    pgm = tmp_path / "pgm"
    pgm.mkdir()
    codes = z["codes"]
    for k in range(nz):
        (pgm / f"v1_{k + 1:05d}.pgm").write_text("P2\n# test\n1 1\n255\n" + " ".join(map(str, codes[k].reshape(-1))))
    p = po.OracleParams()
    p.nx, p.ny, p.nz = nx, ny, nz
    got_codes, specs, sigma, eps_s, eps_i, tau = po.load_materials(p, tmp_path / "mat_specs", pgm, "f64")
    assert np.array_equal(got_codes, codes)
    for got, key in zip((sigma, eps_s, eps_i, tau), ("sigma", "eps_s", "eps_i", "tau")):
        assert bits_equal(got, z[key]), key
    # the record after the comment line was never read
    assert not np.any(specs[40])


def test_oracle_snapshot_text_matches_reference(golden, tmp_path):
    rec = json.loads((golden / "snapshot.json").read_text())
    f = np.load(golden / "snapshot_fields.npz")
    fields = [f[f"arr_{k}"] for k in range(9)]
    po.write_snapshot3d(tmp_path, fields, rec["iteration"], "f64")
    got = {p.name: p.read_text() for p in sorted(tmp_path.iterdir())}
    assert got == rec["files"]


def test_mur_slabs_match_closed_form():
    """The C99-complex restatement of setupMurBoundary against its closed
    form: Re(eps_i + d/(1 + w) - s) for the x slabs (real w, s) and
    eps_i + d/(1 + w^2) for the y and z slabs (w, s times i)."""
    p = po.OracleParams()
    p.nx, p.ny, p.nz = 4, 5, 6
    p.pi, p.wave_frequency, p.eps0 = np.float32(np.pi), 9e8, np.float32(8.841941e-12)
    rng = np.random.default_rng(0)
    sh = (p.nz, p.ny, p.nx)
    sig, es, ei = (rng.uniform(0, 2, sh).astype(np.float32), rng.uniform(10, 80, sh).astype(np.float32),
                   rng.uniform(4, 9, sh).astype(np.float32))
    tau = rng.uniform(0, 5e-10, sh).astype(np.float32)
    rp = po.setup_mur(p, sig, es, ei, tau)
    w = 2 * np.float64(p.pi) * np.float64(p.wave_frequency) * tau.astype(np.float64)
    s = sig.astype(np.float64) / (2 * np.float64(p.pi) * np.float64(p.wave_frequency) * np.float64(p.eps0))
    d = (es - ei).astype(np.float64)
    rx = ei + d / (1 + w) - s
    ryz = ei + d / (1 + w ** 2)
    np.testing.assert_allclose(rp[0][..., 0], rx[:, :, 0], rtol=2e-6)
    np.testing.assert_allclose(rp[3][..., 1], rx[:, :, -1], rtol=2e-6)
    np.testing.assert_allclose(rp[1][:, 0, :], ryz[:, 0, :], rtol=2e-6)
    np.testing.assert_allclose(rp[5][1], ryz[-1], rtol=2e-6)
    # the shipped default material (vacuum) gives exactly 1
    one = po.setup_mur(p, *(np.full(sh, v, np.float32) for v in (0.0, 1.0, 1.0, 0.0)))
    assert all(np.all(r == 1.0) for r in one)


@pytest.mark.skipif(not obuild.reference_available(), reason="reference sources not present")
@pytest.mark.parametrize("seed", [1, 2])
def test_fp32_oracle_matches_reference_kernels_on_random_cases(seed):
    nx, ny, nz = [(23, 7, 13), (9, 31, 6)][seed - 1]
    codes, specs, rp, sources, consts, jz = random_case(nx, ny, nz, seed, nsrc=4)
    media = class_media(codes, specs, rp)
    cfg = po.make_cfg((nx, ny, nz), jz, sources=sources, consts=consts)
    a = po.State(nx, ny, nz, np.float32)
    b = po.State(nx, ny, nz, np.float32)
    po.run(cfg, media, a, 0, 15)
    po.ref_cpu_run(cfg, media, b, 0, 15)
    for x, y in zip(a.arrays(), b.arrays()):
        assert bits_equal(x, y)


def test_reference_scheme_doubles_vacuum_field_every_step():
    """In vacuum the reference's Debye update has c*d = 2, so once the source
    has passed, |E| doubles per step; the corrected scheme stays bounded."""
    n = 12
    media = po.Media(*(np.full((n, n, n), v, np.float32) for v in (0.0, 1.0, 1.0, 0.0)))
    media.rp = [np.ones(s, np.float32) for s in po.rp_shapes(n, n, n)]
    consts = dict(dt=1.9245009e-12, dx=1e-3, dy=1e-3, dz=1e-3, mu0=1.2566371e-06, eps0=8.841941e-12)
    jz = np.zeros(64, np.float32)
    jz[0] = 1.0
    norms = {}
    for corrected in (False, True):
        cfg = po.make_cfg((n, n, n), jz, sources=[(6, 6, 6)], consts=consts, corrected=corrected)
        st = po.State(n, n, n, np.float64)
        out = []
        for k in range(30):
            po.run(cfg, media, st, k, 1)
            out.append(sum(np.abs(a).sum() for a in st.e[k % 3]))
        norms[corrected] = out
    ratio = norms[False][29] / norms[False][28]
    assert 1.9 < ratio < 2.1
    assert norms[True][29] < 10 * max(norms[True][:5])
