"""Generates ``c3_fp64.npz``: the FP64 oracle on the 512 x 512 x 400
precision-form workload, the accuracy reference of the 16-bit-R form.

Workload (the same inputs the GPU side builds): the seeded 8-shell nested
ellipsoid phantom of ``fdtd_gb300.phantom.c2_config`` at 512 x 512 x 400,
its three-cell 900 MHz Ez dipole 20 cells outside the outer shell, Mur faces,
corrected scheme (the reference scheme doubles |E| every step in vacuum),
dt = 0.99 of the Courant limit, 3000 steps.  Inputs go through the oracle's
own readers: input_params (``oracle_params_read`` + the timeskip), the jz
table (``oracle_setup_sources``), the mat_specs records
(``oracle_read_specs``) and Mur slabs from the default material
(``oracle_setup_mur``).

Recorded, as the precision form is specified:
* the E series (3 components, every step) at 16 probe cells drawn with seed
  2024 from the tissue (class > 0, two cells clear of every face);
* the running DFT at the source's 900 MHz (every 5th step, phase
  exp(-i 2 pi f m dt), weight 5 dt) over the 32 planes z = 184 .. 215,
  stored as |E| on every 4th cell in x and y;
* the peak spectral SAR sigma |E|^2 / (2 rho), rho = 1000 kg/m^3, over those
  32 planes at full resolution, and its cell.

Run once on a CPU host (about 20 GB of memory; the oracle runs on every
core): ``python tests/golden/make_c3_fixture.py``.  The output is a fixture:
nothing at test time runs this script.
"""
from __future__ import annotations

import argparse
import hashlib
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from fdtd_gb300 import phantom as ph  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

SHAPE = (400, 512, 512)   # (nz, ny, nx)
STEPS = 3000
TIMESKIP = 0.99
NPROBES, PROBE_SEED = 16, 2024
DFT_STRIDE, DFT_PLANES, SUB = 5, 32, 4
RHO = 1000.0


def probe_cells(codes: np.ndarray, n: int = NPROBES, seed: int = PROBE_SEED) -> list[tuple[int, int, int]]:
    """n seeded tissue cells (class > 0) at least 2 cells from every face; (x, y, z)."""
    nz, ny, nx = codes.shape
    inner = np.zeros(codes.shape, bool)
    inner[2:nz - 2, 2:ny - 2, 2:nx - 2] = True
    cand = np.flatnonzero((codes > 0) & inner)
    pick = np.random.default_rng(seed).choice(cand, size=n, replace=False)
    z, rem = np.divmod(pick, ny * nx)
    y, x = np.divmod(rem, nx)
    return [(int(a), int(b), int(c)) for a, b, c in zip(x, y, z)]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=STEPS)
    ap.add_argument("--out", default=str(HERE / "c3_fp64.npz"))
    args = ap.parse_args()
    nz, ny, nx = SHAPE
    codes, mats, cfg = ph.c2_config(SHAPE)
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        cfg.env_dir, cfg.output_dir = str(tmp / "pgm"), str(tmp / "out")
        ph.write_input_params(tmp / "input_params", cfg)
        ph.write_mat_specs(tmp / "mat_specs", mats)
        q = po.params_read(tmp / "input_params", "f64")
        po.set_timeskip(q, TIMESKIP)
        specs = po.read_specs(tmp / "mat_specs")[: len(mats)]
    jz = po.setup_sources(q)
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    shape = (nz, ny, nx)
    default = [np.full(shape, v, np.float32) for v in (q.default_sigma, q.default_eps_s, q.default_eps_i,
                                                       q.default_tau_d)]
    media.rp = po.setup_mur(q, *default)
    del default
    run_cfg = po.make_cfg(q, jz, corrected=True)
    probes = probe_cells(codes)
    freq = float(q.wave_frequency) * float(q.pulse_modulation_frequency)
    z0 = nz // 2 - DFT_PLANES // 2
    dt = float(q.dt)

    st = po.State(nx, ny, nz, np.float64)
    series = np.zeros((args.steps, NPROBES, 3))
    px, py, pz = (np.array(v) for v in zip(*probes))
    dft = [np.zeros((DFT_PLANES, ny, nx), complex) for _ in range(3)]
    t0 = time.time()
    for k in range(args.steps):
        po.run(run_cfg, media, st, k, 1)
        e = st.e[k % 3]
        for c in range(3):
            series[k, :, c] = e[c][pz, py, px]
        m = k + 1
        if m % DFT_STRIDE == 0:
            w = np.exp(-1j * 2 * np.pi * freq * m * dt) * DFT_STRIDE * dt
            for c in range(3):
                dft[c] += e[c][z0:z0 + DFT_PLANES] * w
        if m % 50 == 0 or m == args.steps:
            print(f"step {m}/{args.steps}  {time.time() - t0:.0f} s", flush=True)
    amp = np.sqrt(sum(np.abs(a) ** 2 for a in dft))
    sig = specs[codes[z0:z0 + DFT_PLANES], 0].astype(np.float64)
    sar = sig * amp ** 2 / (2 * RHO)
    peak = int(np.argmax(sar))
    pk, prem = divmod(peak, ny * nx)
    pyy, pxx = divmod(prem, nx)
    np.savez_compressed(
        args.out,
        shape=np.array(SHAPE), steps=np.int64(args.steps), timeskip=np.float32(TIMESKIP),
        dt=np.float32(q.dt), corrected=np.int64(1), probes=np.array(probes, np.int64),
        series=series.astype(np.float32), dft_hz=np.float64(freq), dft_stride=np.int64(DFT_STRIDE),
        dft_z0=np.int64(z0), dft_planes=np.int64(DFT_PLANES), dft_sub=np.int64(SUB),
        dft_abs_e_sub=amp[:, ::SUB, ::SUB].astype(np.float32), dft_abs_e_norm=np.float64(np.linalg.norm(amp)),
        peak_sar=np.float64(sar.flat[peak]), peak_sar_cell=np.array([pxx, pyy, z0 + pk], np.int64),
        rho=np.float64(RHO), specs=specs, codes_sha256=np.array(hashlib.sha256(codes.tobytes()).hexdigest()),
        jz_head=jz[:4096].copy(), sources=np.array(q.source_list(), np.int64))
    print("wrote", args.out, f"in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
