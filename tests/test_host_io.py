"""Host set-up of the library against the reference's golden outputs."""
from __future__ import annotations

import json

import numpy as np
import pytest

import fdtd_gb300 as fg
from fdtd_gb300 import phantom as ph
from oracle import pyoracle as po

from .helpers import bits_equal


@pytest.mark.parametrize("case", ["vacuum3ghz", "sphere1ghz", "debye900"])
def test_params_and_source_table_bit_exact(golden, tmp_path, case):
    rec = json.loads((golden / f"params_{case}.json").read_text())
    path = tmp_path / "input_params"
    path.write_text(rec["input_params"])
    p = fg.Params.read(path)
    names = {"iterations": "iterationsCount", "elements_per_wave": "elementsPerWave", "wave_frequency": "waveFrequency",
             "pulse_width": "pulseWidth", "pulse_modulation_frequency": "pulseModulationFrequency",
             "nsources": "sourcesCount", "default_sigma": "defaultSigma", "default_eps_s": "defaultEpsS",
             "default_eps_i": "defaultEpsI", "default_tau_d": "defaultTauD"}
    for k, v in rec["params"].items():
        got = getattr(p.raw, names.get(k, k))
        if k in rec["params_f32_hex"]:
            assert np.float32(got).view(np.uint32) == rec["params_f32_hex"][k], k
        else:
            assert got == v, k
    assert [list(s) for s in p.sources] == rec["sources"]
    assert p.inputPath.decode() == rec["input_path"] and p.outputPath.decode() == rec["output_path"]
    jz = p.setup_sources()
    want = np.load(golden / f"jz_{case}.npy")
    assert jz.size == fg.JZ_LEN
    assert bits_equal(jz[: want.size], want)
    assert not np.any(jz[want.size:1 << 14])


def _write_golden_phantom(golden, tmp_path):
    z = np.load(golden / "materials.npz")
    nx, ny, nz = (int(v) for v in z["dims"])
    (tmp_path / "mat_specs").write_text(str(z["specs_text"]))
    pgm = tmp_path / "pgm"
    pgm.mkdir()
    rng = np.random.default_rng(5)
    for k in range(nz):
        vals = [str(v) for v in z["codes"][k].reshape(-1)]
        seps = rng.choice([" ", "\n", "\t", "  \n "], size=len(vals))
        body = "".join(v + s for v, s in zip(vals, seps))
        (pgm / f"v1_{k + 1:05d}.pgm").write_text("P2\n# test\n265 490\n93\n" + body)
    cfg = ph.Config(nx, ny, nz, 3, env_dir=str(pgm), sources=[(1, 1, 1)])
    ph.write_input_params(tmp_path / "input_params", cfg)
    return z, fg.Params.read(tmp_path / "input_params"), pgm


def test_load_materials_bit_exact(golden, tmp_path):
    z, p, pgm = _write_golden_phantom(golden, tmp_path)
    sigma, eps_s, eps_i, tau = fg.load_materials(p, tmp_path / "mat_specs", pgm)
    for got, key in zip((sigma, eps_s, eps_i, tau), ("sigma", "eps_s", "eps_i", "tau")):
        assert bits_equal(got, z[key]), key
    codes = fg.load_material_codes(p, pgm, nthreads=3)
    assert np.array_equal(codes, z["codes"])
    specs = fg.read_specs(tmp_path / "mat_specs")
    assert not np.any(specs[40])  # after the comment line: never read
    assert bits_equal(specs[codes, 0], z["sigma"])


def test_specs_code_94_and_stop(tmp_path):
    """Code 94 is stored (the reference writes it past its 94x4 buffer) and
    ends the record loop; later records are ignored."""
    (tmp_path / "s").write_text("0 air 0 1 1 0\n94 gland 0.8 60.5 27.7 1.77e-11\n95 late 1 2 3 4\n")
    specs = fg.read_specs(tmp_path / "s")
    np.testing.assert_array_equal(specs[94], np.float32([0.8, 60.5, 27.7, 1.77e-11]))
    assert not np.any(specs[95])


def test_loader_errors(tmp_path):
    cfg = ph.Config(4, 3, 2, 3, env_dir=str(tmp_path / "pgm"), sources=[(1, 1, 0)])
    ph.write_input_params(tmp_path / "ip", cfg)
    p = fg.Params.read(tmp_path / "ip")
    with pytest.raises(fg.FdtdError) as e:
        fg.load_material_codes(p, tmp_path / "pgm")
    assert e.value.status == fg.FDTD_ERR_IO
    (tmp_path / "pgm").mkdir()
    for k in (1, 2):
        (tmp_path / "pgm" / f"v1_{k:05d}.pgm").write_text("P2\n# test\n4 3\n1\n" + " 1" * 11)
    with pytest.raises(fg.FdtdError) as e:
        fg.load_material_codes(p, tmp_path / "pgm")
    assert e.value.status == fg.FDTD_ERR_FORMAT
    (tmp_path / "pgm" / "v1_00001.pgm").write_text("P2\n# test\n4 3\n1\n" + " 300" * 12)
    with pytest.raises(fg.FdtdError):
        fg.load_material_codes(p, tmp_path / "pgm")
    with pytest.raises(fg.FdtdError) as e:
        fg.Params.read(tmp_path / "missing")
    assert e.value.status == fg.FDTD_ERR_IO
    (tmp_path / "bad").write_text("nx_ny_nz: 4 3\n")
    with pytest.raises(fg.FdtdError) as e:
        fg.Params.read(tmp_path / "bad")
    assert e.value.status == fg.FDTD_ERR_FORMAT


def test_snapshot_writer_bytes_match_reference(golden, tmp_path):
    rec = json.loads((golden / "snapshot.json").read_text())
    f = np.load(golden / "snapshot_fields.npz")
    nx, ny, nz = rec["dims"]
    cfg = ph.Config(nx, ny, nz, 3, output_dir=str(tmp_path), sources=[(1, 1, 0)])
    ph.write_input_params(tmp_path / "ip", cfg)
    p = fg.Params.read(tmp_path / "ip")
    fields = {n: f[f"arr_{k}"] for k, n in enumerate(fg.FIELDS)}
    fg.write_results3d(p, fields, rec["iteration"], nthreads=4)
    got = {q.name: q.read_text() for q in sorted(tmp_path.glob("*_field_*.out"))}
    assert got == rec["files"]


def test_snapshot_writer_fast_path_matches_printf(tmp_path):
    """Many random magnitudes, including values a hair from rounding ties."""
    rng = np.random.default_rng(9)
    nx, ny, nz = 257, 3, 1
    v = (rng.standard_normal(nx * ny) * 10.0 ** rng.integers(-38, 38, nx * ny)).astype(np.float32)
    ties = np.float32([1.0005, 2.5005e3, 9.9995, 1.2345e-3, 6.5e-7, 1.0e10, 0.1, 0.3, 123.45, 99995.0])
    v[: ties.size] = ties
    cfg = ph.Config(nx, ny, nz, 3, output_dir=str(tmp_path), sources=[(1, 1, 0)])
    ph.write_input_params(tmp_path / "ip", cfg)
    p = fg.Params.read(tmp_path / "ip")
    fg.write_results3d(p, {"ex": v.reshape(nz, ny, nx)}, 0)
    text = (tmp_path / "E_field_x_00000_z00000.out").read_text()
    want = "".join("".join(" % 9.3E" % float(x) for x in row) + "\n" for row in v.reshape(ny, nx))
    assert text == want


def test_mur_slabs_match_oracle():
    p = fg.Params.__new__(fg.Params)
    raw = fg.FdtdParams()
    raw.nx, raw.ny, raw.nz = 6, 5, 4
    raw.pi, raw.waveFrequency, raw.eps0 = np.float32(np.pi), 9e8, np.float32(8.841941e-12)
    p.raw = raw
    rng = np.random.default_rng(2)
    sh = (4, 5, 6)
    arrs = [rng.uniform(0, 2, sh), rng.uniform(10, 80, sh), rng.uniform(4, 9, sh), rng.uniform(0, 2e-9, sh)]
    arrs = [a.astype(np.float32) for a in arrs]
    rp = fg.setup_mur(p, *arrs)
    q = po.OracleParams()
    q.nx, q.ny, q.nz, q.pi, q.wave_frequency, q.eps0 = 6, 5, 4, raw.pi, raw.waveFrequency, raw.eps0
    want = po.setup_mur(q, *arrs)
    for a, b in zip(rp, want):
        assert bits_equal(a, b)
    uni = fg.setup_mur_uniform(p, 0.5, 50.0, 4.0, 8e-12)
    full = fg.setup_mur(p, *(np.full(sh, v, np.float32) for v in (0.5, 50.0, 4.0, 8e-12)))
    for a, b in zip(uni, full):
        assert bits_equal(a, b)
    p.raw = None


def test_timeskip_rederives_dt(tmp_path):
    cfg = ph.Config(8, 8, 8, 3, sources=[(2, 2, 2)])
    ph.write_input_params(tmp_path / "ip", cfg)
    p = fg.Params.read(tmp_path / "ip")
    dt1 = p.dt
    p.set_timeskip(0.99)
    assert p.timeskip == np.float32(0.99)
    np.testing.assert_allclose(p.dt, 0.99 * dt1, rtol=1e-6)


def test_phantom_writer_round_trip(tmp_path):
    path = ph.c1_inputs(tmp_path, n=16, t_max=10)
    p = fg.Params.read(path)
    assert (p.nx, p.ny, p.nz, p.iterationsCount) == (16, 16, 16, 12)
    assert p.sources == [(4, 8, 8)]
    codes = fg.load_material_codes(p, tmp_path / "pgm")
    assert np.array_equal(codes, ph.sphere_phantom(16, 4.0))
    specs = fg.read_specs(tmp_path / "mat_specs")
    np.testing.assert_array_equal(specs[1], np.float32([0.5, 50.0, 4.0, 8e-12]))


def test_voxel_cache_hit_miss_and_invalidation(golden, tmp_path):
    """The first load parses the slices and writes the cache; the second reads
    the cache; touching a slice (new size or time) or asking for other
    dimensions makes it parse again.  Every load equals the parsed volume."""
    import os

    z, p, pgm = _write_golden_phantom(golden, tmp_path)
    cache = tmp_path / "codes.u8v"
    codes, hit = fg.load_material_codes_cached(p, pgm, cache)
    assert not hit and cache.exists()
    assert np.array_equal(codes, z["codes"])
    assert cache.stat().st_size == 32 + codes.size
    codes, hit = fg.load_material_codes_cached(p, pgm, cache, nthreads=2)
    assert hit and np.array_equal(codes, z["codes"])
    assert np.array_equal(fg.load_material_codes(p, pgm, cache=cache), z["codes"])
    # a slice rewritten with another class: its time changes, so the cache is stale
    first = sorted(pgm.iterdir())[0]
    text = first.read_text()
    lines = text.split("\n")
    body = " ".join(lines[4:]).split()
    body[0] = "0" if body[0] != "0" else "1"
    first.write_text("\n".join(lines[:4]) + "\n" + " ".join(body) + "\n")
    st = first.stat()
    os.utime(first, ns=(st.st_atime_ns, st.st_mtime_ns + 1_000_000_000))
    codes, hit = fg.load_material_codes_cached(p, pgm, cache)
    assert not hit
    assert np.array_equal(codes, fg.load_material_codes(p, pgm))
    assert not np.array_equal(codes, z["codes"])
    # a truncated cache is a miss, never an error
    cache.write_bytes(cache.read_bytes()[:40])
    codes2, hit = fg.load_material_codes_cached(p, pgm, cache)
    assert not hit and np.array_equal(codes2, codes)
    _, hit = fg.load_material_codes_cached(p, pgm, cache)
    assert hit
    # an unwritable cache path still loads
    codes3, hit = fg.load_material_codes_cached(p, pgm, tmp_path / "no_dir" / "c.u8v")
    assert not hit and np.array_equal(codes3, codes)
