"""The compact forms' strip kernel (TMA loads and stores over column strips,
fdtd_gb300/csrc/step_strip.cu) against the z-marching kernel it replaces
wherever rows are a multiple of 16 cells: both apply the same arithmetic
(cell_math.cuh), so every field must agree bit for bit after many steps, on
grids with partial tiles in y and z, interior tiles (the path without range
tests) and edge tiles, sources on tile borders and on the cells next to the
faces, tile-planes of vacuum only (whose R the strip kernel neither reads nor
writes), both schemes and both storage forms (32-bit R and 16-bit R).  The
z-marching kernel is itself held to the oracle by the other tests, and the
strip kernel runs in every compact-form test whose rows allow it."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg

from .gpu_util import Params, make_params
from .helpers import random_case

pytestmark = pytest.mark.gpu

CASES = [
    ((32, 9, 7), 24),      # one tile column, partial tile rows, one z chunk
    ((64, 24, 40), 30),    # x faces in every tile, three z chunks
    ((96, 37, 21), 30),    # one interior tile column, partial rows
    ((128, 72, 53), 40),   # interior tiles in x and y, four z chunks
    ((48, 3, 3), 12),      # the smallest grid
]


def _run(p, codes, specs, scheme, kernel, steps):
    with fg.Solver(p, codes, specs, scheme=scheme, kernel=kernel, nclasses=len(specs)) as s:
        s.run(steps)
        out = s.fields()
        names = set(s.profile(1))
    return out, names


@pytest.mark.parametrize("shape", [0, 1, 2, 3])
@pytest.mark.parametrize("kernel", [fg.KERNEL_COMPACT, fg.KERNEL_COMPACT_R16])
@pytest.mark.parametrize("scheme", [fg.SCHEME_REFERENCE, fg.SCHEME_CORRECTED])
@pytest.mark.parametrize("dims,steps", CASES)
def test_strip_kernel_equals_z_marching_kernel(cuda, monkeypatch, dims, steps, scheme, kernel, shape):
    """Every strip shape (FDTD_STRIP_SHAPE: 8-row tiles of 2 x 4, 1 x 8 and
    4 x 2 cells per thread x warps, 16-row tiles of 4 x 4)."""
    nx, ny, nz = dims
    codes, specs, rp, sources, consts, jz = random_case(nx, ny, nz, seed=nx + ny + nz, ncls=6, nsrc=2)
    # vacuum (class 0, tau = 0) in the lower half of y and in a block of
    # planes: tile-planes without Debye memory, whose R the strip kernel skips
    codes[:, : ny // 2, :] = 0
    codes[nz // 3: nz // 2] = 0
    # sources on tile borders (x = 31 | 32, y = 7 | 8, z on a chunk border)
    # and next to the low faces, where they fit the grid
    extra = [(min(31, nx - 2), min(8, ny - 2), min(16, nz - 1)), (min(32, nx - 1), min(7, ny - 1), min(15, nz - 1)),
             (1, 1, 0), (nx - 1, ny - 1, nz - 1)]
    sources = (sources + extra)[: fg.MAX_SOURCES]
    raw = make_params(dims, consts, sources, jz)
    p = Params(raw)
    monkeypatch.setenv("FDTD_COMPACT_STEP", "zmarch")
    want, _ = _run(p, codes, specs, scheme, kernel, steps)
    monkeypatch.delenv("FDTD_COMPACT_STEP")
    monkeypatch.setenv("FDTD_STRIP_SHAPE", str(shape))
    got, names = _run(p, codes, specs, scheme, kernel, steps)
    assert names == {"compact16_step" if kernel == fg.KERNEL_COMPACT_R16 else "compact_step", "mur"}
    assert sorted(got) == sorted(want)
    for name in want:
        a, b = got[name], want[name]
        same = a.view(np.uint32) == b.view(np.uint32)
        if not same.all():
            z, y, x = np.argwhere(~same)[0]
            raise AssertionError(f"{name} differs at x={x} y={y} z={z}: {a[z, y, x]!r} vs {b[z, y, x]!r} "
                                 f"({(~same).sum()} cells)")
