"""The 16-bit-R form (FDTD_KERNEL_COMPACT_R16) against the FP64 oracle on a
scaled-down nested-ellipsoid Debye phantom: the 512x512x400 benchmark
phantom's recipe at 96x96x75 cells (semi-axes scaled by 96/512, so several
tissue shells remain), its 900 MHz three-cell dipole outside the outer shell,
corrected scheme, 1500 steps.  Compared, as the precision form is specified:
the E series at 16 seeded probe points inside the tissue, the running DFT
|E| at 900 MHz over 32 planes through the source, and the peak spectral SAR
over those planes (rho 1000 kg/m^3).  The FP32 D form is held to the same
comparison for scale."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from fdtd_gb300 import phantom as ph
from oracle import pyoracle as po

from .helpers import rel_l2

pytestmark = pytest.mark.gpu

R16_TOL = 1e-3
NX, NY, NZ = 96, 96, 75
STEPS, STRIDE, NPROBES = 1500, 5, 16


def _phantom(root):
    s = NX / 512.0
    codes, mats, outer = ph.ellipsoid_phantom((NZ, NY, NX), seed=0, semi_min=60.0 * s, semi_max=230.0 * s)
    cx, cy, cz = (NX - 1) // 2, (NY - 1) // 2, (NZ - 1) // 2
    sx = max(int(round(cx - outer[0] - 4)), 1)
    cfg = ph.Config(NX, NY, NZ, STEPS, wave_frequency=1.0e9, elements_per_wavelength=300, pulse_width=0.5,
                    pulse_modulation_frequency=0.9, sources=[(sx, cy, cz + d) for d in (-1, 0, 1)],
                    env_dir=str(root / "pgm"), output_dir=str(root / "out"))
    ph.write_input_params(root / "input_params", cfg)
    ph.write_mat_specs(root / "mat_specs", mats)
    p = fg.Params.read(root / "input_params")
    p.set_timeskip(0.99)
    specs = fg.read_specs(root / "mat_specs")[: len(mats)]
    return p, codes, specs


def _probes(codes):
    inner = np.zeros(codes.shape, bool)
    inner[2:-2, 2:-2, 2:-2] = True
    cand = np.flatnonzero((codes > 0) & inner)
    pick = np.random.default_rng(7).choice(cand, size=NPROBES, replace=False)
    z, rem = np.divmod(pick, NY * NX)
    y, x = np.divmod(rem, NX)
    return [(int(a), int(b), int(c)) for a, b, c in zip(x, y, z)]


def test_compact16_probes_dft_and_sar_vs_fp64_oracle(cuda, tmp_path):
    p, codes, specs = _phantom(tmp_path)
    assert len(np.unique(codes)) >= 4  # vacuum and at least three tissue shells
    probes = _probes(codes)
    freq = float(p.waveFrequency) * float(p.pulseModulationFrequency)
    z0, npl = NZ // 2 - 16, 32
    dt = float(p.dt)

    got = {}
    for kernel in (fg.KERNEL_COMPACT_R16, fg.KERNEL_SINGLE_PASS):
        with fg.Solver(p, codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel) as s:
            s.set_probes(probes, capacity=STEPS)
            s.set_dft(freq, stride=STRIDE, z0=z0, nplanes=npl)
            s.run(STEPS)
            acc = [s.dft(c) for c in range(3)]
            got[kernel] = (s.probes().astype(np.float64), np.sqrt(sum(np.abs(a) ** 2 for a in acc)),
                           s.peak_sar()[0])

    # FP64 oracle, step by step, the same probe points and DFT rule
    q = po.params_read(tmp_path / "input_params", "f64")
    q.dt = p.dt
    jz = p.setup_sources()
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    media.rp = po.uniform_media(q).rp
    cfg = po.make_cfg(q, jz, corrected=True)
    st = po.State(NX, NY, NZ, np.float64)
    series = np.zeros((STEPS, NPROBES, 3))
    pz, py, px = (np.array(v) for v in zip(*[(z, y, x) for x, y, z in probes]))
    dft = [np.zeros((npl, NY, NX), complex) for _ in range(3)]
    for k in range(STEPS):
        po.run(cfg, media, st, k, 1)
        e = st.e[k % 3]
        for c in range(3):
            series[k, :, c] = e[c][pz, py, px]
        m = k + 1
        if m % STRIDE == 0:
            ph_ = np.exp(-1j * 2 * np.pi * freq * m * dt) * STRIDE * dt
            for c in range(3):
                dft[c] += e[c][z0:z0 + npl] * ph_
    amp = np.sqrt(sum(np.abs(a) ** 2 for a in dft))
    sig = specs[codes[z0:z0 + npl], 0].astype(np.float64)
    sar = (sig * amp ** 2 / (2 * 1000.0)).max()

    report = {}
    for kernel, name in ((fg.KERNEL_COMPACT_R16, "compact16"), (fg.KERNEL_SINGLE_PASS, "d_form")):
        ser, a, peak = got[kernel]
        per = [rel_l2(ser[:, j], series[:, j]) for j in range(NPROBES)]
        report[name] = (max(per), float(np.median(per)), rel_l2(a, amp), abs(peak - sar) / sar)
    print("precision vs FP64 oracle (probe max, probe median, DFT |E|, peak SAR):", report)
    assert max(report["compact16"]) <= R16_TOL, report
    assert max(report["d_form"]) <= R16_TOL, report
