"""The storage forms against the FP64 oracle on the full precision-form
workload: the 512 x 512 x 400 nested-ellipsoid Debye phantom (8 shells), its
900 MHz three-cell dipole, corrected scheme, dt = 0.99 of the Courant limit,
3000 steps, compared with the FP64 oracle's record of the same run
(tests/golden/c3_fp64.npz, made by tests/golden/make_c3_fixture.py):

* the E series at 16 seeded probe cells inside the tissue (relative L2 per
  probe over the three components and all steps) -- the form's stated
  tolerance, 1e-3;
* the running DFT |E| at 900 MHz over 32 planes through the source (on every
  4th cell in x and y, as recorded);
* the peak spectral SAR over those planes (rho 1000 kg/m^3) and its cell.

The inputs are rebuilt here from the same seeded generator and checked
against the record (class volume hash, class table, dt) before any
comparison."""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np
import pytest

import fdtd_gb300 as fg
from fdtd_gb300 import phantom as ph

from .helpers import rel_l2

FIXTURE = Path(__file__).resolve().parent / "golden" / "c3_fp64.npz"
pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not FIXTURE.exists(), reason="FP64 record not generated")]

PROBE_TOL = 1e-3   # the precision form's tolerance on every probe's E series
DFT_TOL = 1e-4     # DFT |E| over the recorded cells
SAR_TOL = 1e-3     # peak spectral SAR


def _inputs(f, root: Path):
    nz, ny, nx = (int(v) for v in f["shape"])
    codes, mats, cfg = ph.c2_config((nz, ny, nx))
    assert hashlib.sha256(codes.tobytes()).hexdigest() == str(f["codes_sha256"])
    cfg.env_dir, cfg.output_dir = str(root / "pgm"), str(root / "out")
    ph.write_input_params(root / "input_params", cfg)
    ph.write_mat_specs(root / "mat_specs", mats)
    p = fg.Params.read(root / "input_params")
    p.set_timeskip(float(f["timeskip"]))
    assert np.float32(p.dt) == f["dt"]
    specs = fg.read_specs(root / "mat_specs")[: len(mats)]
    assert np.array_equal(specs, f["specs"])
    assert np.array_equal(p.setup_sources()[: f["jz_head"].size], f["jz_head"])
    return p, codes, specs


@pytest.mark.parametrize("kernel", [fg.KERNEL_COMPACT_R16, fg.KERNEL_COMPACT])
def test_storage_forms_vs_fp64_oracle_on_the_full_phantom(cuda, tmp_path, kernel):
    f = np.load(FIXTURE)
    p, codes, specs = _inputs(f, tmp_path)
    steps, sub = int(f["steps"]), int(f["dft_sub"])
    probes = [tuple(int(v) for v in r) for r in f["probes"]]
    z0, npl = int(f["dft_z0"]), int(f["dft_planes"])
    with fg.Solver(p, codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel) as s:
        s.set_probes(probes, capacity=steps)
        s.set_dft(float(f["dft_hz"]), stride=int(f["dft_stride"]), z0=z0, nplanes=npl)
        s.run(steps)
        series = s.probes().astype(np.float64)
        amp = np.sqrt(sum(np.abs(s.dft(c)) ** 2 for c in range(3)))
        sar, cell = s.peak_sar()
    ref = f["series"].astype(np.float64)
    per = [rel_l2(series[:, j], ref[:, j]) for j in range(len(probes))]
    dft = rel_l2(amp[:, ::sub, ::sub], f["dft_abs_e_sub"].astype(np.float64))
    sar_err = abs(sar - float(f["peak_sar"])) / float(f["peak_sar"])
    nz, ny, nx = codes.shape
    pc = f["peak_sar_cell"]
    same_cell = cell == int((pc[2] * ny + pc[1]) * nx + pc[0])
    print(f"kernel {kernel}: probes max {max(per):.3e} median {np.median(per):.3e}, DFT |E| {dft:.3e}, "
          f"peak SAR {sar_err:.3e} (same cell: {same_cell})")
    assert max(per) <= PROBE_TOL, per
    assert dft <= DFT_TOL
    assert sar_err <= SAR_TOL and same_cell
