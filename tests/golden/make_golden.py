"""Generates the golden fixtures in this directory from the reference itself.

Run where the reference sources are, naming their directory:
``FDTD_REFERENCE_ROOT=<dir> python tests/golden/make_golden.py``.  It builds
oracle/_ref (the reference's own host code and its kernels compiled for the
CPU) and records their outputs on synthetic inputs:

* ``params_<case>.json`` + ``jz_<case>.npy``: initParamsWithPath and
  setupSources on generated input_params files (inputs stored in the JSON);
* ``materials.npz``: loadMaterials on a generated phantom whose mat_specs file
  has a comment line in the middle (records after it are never read);
* ``snapshot.json``: writeResults3d text for fields holding ties, subnormals,
  infinities and NaNs;
* ``run_<case>.npz``: the reference kernels looped with the reference's slot
  rotation, inputs and the final 21-array state.

The fixtures travel with the repository; nothing at test time reads the
reference sources.
"""
from __future__ import annotations

import json
import shutil
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import os  # noqa: E402

if not os.environ.get("FDTD_REFERENCE_ROOT"):
    raise SystemExit("set FDTD_REFERENCE_ROOT to the directory holding the reference sources")

from fdtd_gb300 import phantom as ph  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

PARAM_FIELDS = ["nx", "ny", "nz", "iterations", "elements_per_wave", "wave_frequency", "pulse_width",
                "pulse_modulation_frequency", "nsources", "default_sigma", "default_eps_s", "default_eps_i",
                "default_tau_d", "pi", "c", "timeskip", "lambda_", "dt", "dx", "dy", "dz", "mu0", "eps0"]

PARAM_CASES = {
    "vacuum3ghz": ph.Config(100, 100, 100, 3, elements_per_wavelength=100, wave_frequency=3.0e9,
                            pulse_width=0.5, pulse_modulation_frequency=0.0, sources=[(49, 49, 49)]),
    "sphere1ghz": ph.Config(64, 64, 64, 500, elements_per_wavelength=300, wave_frequency=1.0e9,
                            pulse_width=0.5, pulse_modulation_frequency=1.0, sources=[(16, 32, 32)]),
    "debye900": ph.Config(40, 30, 20, 7, elements_per_wavelength=217, wave_frequency=9.0e8, pulse_width=0.4,
                          pulse_modulation_frequency=0.9, sources=[(3, 4, 5), (39, 29, 19)],
                          default=ph.Material(0, "bg", 0.25, 30.0, 6.0, 9.0e-12)),
}


def _value(v):
    if isinstance(v, bytes):
        return v.decode()
    if isinstance(v, float):
        return float(np.float32(v))
    return v


def params_fixtures(tmp: Path) -> None:
    for name, cfg in PARAM_CASES.items():
        path = tmp / f"input_params_{name}"
        ph.write_input_params(path, cfg)
        p = po.params_read(path, "ref")
        jz = po.setup_sources(p, "ref")
        rec = {"input_params": path.read_text(),
               "params": {k: _value(getattr(p, k)) for k in PARAM_FIELDS},
               "params_f32_hex": {k: np.float32(getattr(p, k)).view(np.uint32).item()
                                  for k in PARAM_FIELDS if isinstance(getattr(p, k), float)},
               "sources": [list(s) for s in p.source_list()],
               "input_path": p.input_path.decode(), "output_path": p.output_path.decode()}
        (HERE / f"params_{name}.json").write_text(json.dumps(rec, indent=1, sort_keys=True))
        np.save(HERE / f"jz_{name}.npy", jz[:2048])
        assert not np.any(jz[2048:16384]), "jz table longer than the stored prefix"


def materials_fixture(tmp: Path) -> None:
    nx, ny, nz = 13, 11, 7
    rng = np.random.default_rng(7)
    mats = [ph.Material(c, f"m{c}", float(rng.uniform(0, 2)), float(rng.uniform(10, 80)),
                        float(rng.uniform(4, 10)), float(rng.uniform(5e-12, 3e-11))) for c in (0, 1, 2, 5, 17, 93)]
    late = [ph.Material(40, "after_comment", 9.0, 9.0, 9.0, 9e-12)]
    specs_text = "\n".join(f"{m.code} {m.name}\t{m.sigma:.8f}\t{m.eps_s:.8f}\t{m.eps_i:.8f}\t{m.tau:.8E}"
                           for m in mats[:4])
    specs_text += "\n! a comment line stops the reference's record loop\n"
    specs_text += "\n".join(f"{m.code} {m.name}\t{m.sigma:.8f}\t{m.eps_s:.8f}\t{m.eps_i:.8f}\t{m.tau:.8E}"
                            for m in mats[4:] + late) + "\n"
    (tmp / "mat_specs").write_text(specs_text)
    codes = rng.choice([0, 1, 2, 5, 17, 93, 40, 3], size=(nz, ny, nx)).astype(np.uint8)
    pgm = tmp / "pgm"
    pgm.mkdir()
    for z in range(nz):
        # irregular line breaks and a header whose W H differ from nx ny
        vals = [str(v) for v in codes[z].reshape(-1)]
        lines, k = [], 0
        while k < len(vals):
            step = int(rng.integers(1, 9))
            lines.append("  ".join(vals[k:k + step]))
            k += step
        (pgm / f"v1_{z + 1:05d}.pgm").write_text("P2\n# test\n265 490\n93\n" + "\n".join(lines) + "\n")
    cfg = ph.Config(nx, ny, nz, 3, env_dir=str(pgm), sources=[(1, 1, 1)])
    ph.write_input_params(tmp / "input_params", cfg)
    p = po.params_read(tmp / "input_params", "ref")
    _, _, sigma, eps_s, eps_i, tau = po.load_materials(p, tmp / "mat_specs", pgm, "ref")
    np.savez_compressed(HERE / "materials.npz", codes=codes, specs_text=np.array(specs_text),
                        sigma=sigma, eps_s=eps_s, eps_i=eps_i, tau=tau, dims=np.array([nx, ny, nz]))


def snapshot_fixture(tmp: Path) -> None:
    nx, ny, nz = 5, 3, 2
    rng = np.random.default_rng(3)
    special = np.array([0.0, -0.0, 1.0625, -2.5, 1e-40, -3e-42, np.inf, -np.inf, np.nan, 9.9995e5, 9.9994e5,
                        1.2345e-7, 3.4e38, -1.17549435e-38, 1.0], np.float32)
    fields = []
    for f in range(9):
        a = rng.standard_normal((nz, ny, nx)).astype(np.float32) * np.float32(10.0 ** rng.integers(-30, 30))
        a.reshape(-1)[:special.size] = np.roll(special, f)[: a.size]
        fields.append(a)
    out = tmp / "snap"
    out.mkdir()
    p = po.OracleParams()
    p.nx, p.ny, p.nz = nx, ny, nz
    po.write_snapshot3d(out, fields, 42, "ref", p)
    files = {f.name: f.read_text() for f in sorted(out.iterdir())}
    np.savez_compressed(HERE / "snapshot_fields.npz", *fields)
    (HERE / "snapshot.json").write_text(json.dumps({"iteration": 42, "dims": [nx, ny, nz], "files": files}))


def run_fixture(name: str, dims, steps: int, media: po.Media, cfg, classes=None) -> None:
    nx, ny, nz = dims
    st = po.State(nx, ny, nz, np.float32)
    po.ref_cpu_run(cfg, media, st, 0, steps)
    arrays = {f"s{i}": a for i, a in enumerate(st.arrays())}
    extra = {}
    if classes is not None:
        extra = {"codes": classes[0], "specs": classes[1]}
    np.savez_compressed(
        HERE / f"run_{name}.npz", dims=np.array(dims), steps=np.array(steps),
        consts=np.array([cfg.dt, cfg.dx, cfg.dy, cfg.dz, cfg.mu0, cfg.eps0], np.float32),
        sources=np.array(cfg._keep[0]).reshape(-1, 3), jz=np.array(cfg._keep[1][:max(steps + 3, 64)]),
        sigma=media.sigma, eps_i=media.eps_i, eps_s=media.eps_s, tau_d=media.tau_d,
        rp=np.concatenate([r.reshape(-1) for r in media.rp]), **arrays, **extra)


def run_fixtures(tmp: Path) -> None:
    # (a) odd grid, per-cell random Debye media, random Mur slabs, sources at
    # an interior cell and on the far x/y faces, 20 steps
    nx, ny, nz = 17, 9, 11
    rng = np.random.default_rng(11)
    sh = (nz, ny, nx)
    m = po.Media(sigma=rng.uniform(0, 2, sh).astype(np.float32), eps_i=rng.uniform(4, 10, sh).astype(np.float32),
                 eps_s=rng.uniform(10, 80, sh).astype(np.float32), tau_d=rng.uniform(5e-12, 15e-12, sh).astype(np.float32))
    m.rp = [rng.uniform(1, 3, s).astype(np.float32) for s in po.rp_shapes(nx, ny, nz)]
    consts = dict(dt=1.9245009e-12, dx=1e-3, dy=1e-3, dz=1e-3, mu0=1.2566371e-06, eps0=8.841941e-12)
    jz = rng.standard_normal(64).astype(np.float32)
    cfg = po.make_cfg((nx, ny, nz), jz, sources=[(3, 4, 5), (16, 8, 10), (15, 7, 0)], consts=consts)
    run_fixture("random17x9x11", (nx, ny, nz), 20, m, cfg)

    # (b) 24^3 sphere case through the reference's own parser and source table
    path = ph.c1_inputs(tmp / "c1", n=24, t_max=60)
    p = po.params_read(path, "ref")
    jz = po.setup_sources(p, "ref")
    codes, specs, sigma, eps_s, eps_i, tau = po.load_materials(p, tmp / "c1" / "mat_specs", tmp / "c1" / "pgm", "f64")
    media = po.Media(sigma=sigma, eps_i=eps_i, eps_s=eps_s, tau_d=tau)
    media.rp = po.uniform_media(p).rp
    cfg = po.make_cfg(p, jz)
    run_fixture("sphere24", (p.nx, p.ny, p.nz), 48, media, cfg, classes=(codes, specs[:2]))

    # (c) class-coded media on a grid wider than one warp, Debye default
    # material for the Mur slabs, two sources, 12 steps
    nx, ny, nz = 70, 20, 9
    ncls = 6
    spec = np.zeros((ncls, 4), np.float32)
    spec[0] = (0.0, 1.0, 1.0, 0.0)
    for k in range(1, ncls):
        spec[k] = (rng.uniform(0.05, 2), rng.uniform(10, 80), rng.uniform(4, 10), rng.uniform(5e-12, 15e-12))
    codes = rng.integers(0, ncls, size=(nz, ny, nx)).astype(np.uint8)
    media = po.Media(sigma=spec[codes, 0].copy(), eps_s=spec[codes, 1].copy(), eps_i=spec[codes, 2].copy(),
                     tau_d=spec[codes, 3].copy())
    pc = ph.Config(nx, ny, nz, 12, elements_per_wavelength=300, wave_frequency=1.0e9, pulse_modulation_frequency=1.0,
                   sources=[(35, 10, 4), (1, 1, 8)], default=ph.Material(0, "bg", 0.3, 20.0, 5.0, 1.0e-11))
    ph.write_input_params(tmp / "input_params_c", pc)
    p = po.params_read(tmp / "input_params_c", "ref")
    jz = po.setup_sources(p, "ref")
    media.rp = po.uniform_media(p).rp
    cfg = po.make_cfg(p, jz)
    run_fixture("classes70x20x9", (nx, ny, nz), 12, media, cfg, classes=(codes, spec))


def main() -> None:
    tmp = Path(tempfile.mkdtemp())
    try:
        params_fixtures(tmp)
        materials_fixture(tmp)
        snapshot_fixture(tmp)
        run_fixtures(tmp)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
