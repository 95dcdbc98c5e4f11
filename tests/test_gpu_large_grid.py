"""A grid of more than 2^31 cells (1300^3 = 2.2e9 cells; 134 GB of state in
the compact form, 160 GB in the D form): all 64-bit index paths.  A source
and a small Debye block sit near the far corner, so the cells around them have
indices beyond 2^31.  For 12 steps the fields there depend only on cells
within reach of the wave, so they must equal those of a 64^3 grid holding
the same local problem at the same position relative to the 32x8 tiles."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg

from .gpu_util import Params, make_params

pytestmark = pytest.mark.gpu

BIG, SMALL = (1300, 1300, 1300), (64, 64, 64)
# source positions: same lane, same row within the tile and, for the D form,
# the same offset within the z chunk (1300 planes make chunks of 62 from 1240;
# 64 planes make one chunk).  The compact form's 16-plane chunks put the
# source at offset 0 (big) and 8 (small); the update of a cell does not depend
# on where the chunk borders lie.
SRC_BIG, SRC_SMALL = (1280, 1280, 1280), (32, 32, 40)
STEPS = 12


def _run(dims, src, kernel):
    nx, ny, nz = dims
    codes = np.zeros((nz, ny, nx), np.uint8)
    x, y, z = src
    codes[z - 3:z + 3, y - 4:y + 2, x - 2:x + 4] = 1  # a Debye block around the source
    specs = np.array([[0.0, 1.0, 1.0, 0.0], [0.5, 40.0, 8.0, 9.0e-12]], np.float32)
    consts = dict(dt=1.9053e-12, dx=1e-3, dy=1e-3, dz=1e-3, mu0=1.2566371e-06, eps0=8.841941e-12)
    jz = np.sin(np.arange(64) * 0.3).astype(np.float32) * 2.0
    raw = make_params(dims, consts, [src], jz)
    probes = [(x + dx, y + dy, z + dz) for dx in (-2, -1, 0, 1) for dy in (-2, -1, 0, 1) for dz in (-2, -1, 0, 1)]
    with fg.Solver(Params(raw), codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel) as s:
        s.set_probes(probes, capacity=STEPS)
        s.run(STEPS)
        return s.probes()


@pytest.mark.parametrize("kernel", [fg.KERNEL_COMPACT, fg.KERNEL_SINGLE_PASS])
def test_grid_beyond_2_31_cells_matches_small_grid(cuda, kernel):
    assert BIG[0] * BIG[1] * BIG[2] > 2 ** 31
    x, y, z = SRC_BIG
    assert (z * BIG[1] + y) * BIG[0] + x > 2 ** 31
    big = _run(BIG, SRC_BIG, kernel)
    small = _run(SMALL, SRC_SMALL, kernel)
    assert big.shape == small.shape == (STEPS, 64, 3)
    assert np.abs(small).max() > 0
    np.testing.assert_allclose(big, small, rtol=1e-6, atol=1e-6 * np.abs(small).max())
