"""Grids at and near the smallest sizes and with partial tiles in every axis
(nx below one 32-column tile or one over a multiple, ny below one 8-row tile,
nz of 3 and just over one z chunk), sources on the face-adjacent cells, for
every kernel kind and both schemes, against the oracle: the FP32 oracle (the
reference kernels) for the reference scheme; the FP64 oracle for the
corrected scheme, where a field may miss 1e-5 only by as much as the
reference's own FP32 arithmetic does on the same case (twice its error)."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from oracle import pyoracle as po

from .gpu_util import Params, make_params
from .helpers import REL_L2_TOL, assert_fields_close, class_media, random_case, rel_l2

pytestmark = pytest.mark.gpu

DIMS = [(3, 3, 3), (5, 4, 3), (33, 7, 5), (31, 9, 66), (64, 17, 65)]
KERNELS = [fg.KERNEL_SINGLE_PASS, fg.KERNEL_COMPACT, fg.KERNEL_TWO_PASS]


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("scheme", [fg.SCHEME_CORRECTED, fg.SCHEME_REFERENCE])
def test_small_and_ragged_grids(cuda, dims, kernel, scheme):
    nx, ny, nz = dims
    steps = 24
    codes, specs, _, _, consts, jz = random_case(*dims, seed=nx * 7 + ny * 3 + nz, ncls=3, nsrc=0)
    # face-adjacent cells and the far corner (x, y >= 1 as the source update reads x-1, y-1)
    sources = [(1, 1, 0), (nx - 1, ny - 1, nz - 1), (max(1, nx // 2), max(1, ny // 2), nz // 2)]
    raw = make_params(dims, consts, sources, jz)
    with fg.Solver(Params(raw), codes, specs, scheme=scheme, kernel=kernel) as s:
        s.run(steps)
        got = s.fields()
    p = po.OracleParams()
    p.nx, p.ny, p.nz = dims
    p.pi, p.wave_frequency, p.eps0 = raw.pi, raw.waveFrequency, raw.eps0
    p.default_sigma, p.default_eps_s = raw.defaultSigma, raw.defaultEpsS
    p.default_eps_i, p.default_tau_d = raw.defaultEpsI, raw.defaultTauD
    media = class_media(codes, specs, po.uniform_media(p).rp)
    corrected = scheme == fg.SCHEME_CORRECTED
    cfg = po.make_cfg(dims, jz, sources=sources, consts=consts, corrected=corrected)
    st = po.State(*dims, np.float64 if corrected else np.float32)
    po.run(cfg, media, st, 0, steps)
    want = st.latest(steps)
    assert all(np.all(np.isfinite(want[k])) for k in got)
    if not corrected:
        assert_fields_close(got, want, names=list(got))
        return
    f32 = po.State(*dims, np.float32)
    po.run(cfg, media, f32, 0, steps)
    ref32 = f32.latest(steps)
    for name in got:
        bound = max(REL_L2_TOL, 2.0 * rel_l2(ref32[name], want[name]))
        assert rel_l2(got[name], want[name]) <= bound, (name, rel_l2(got[name], want[name]), bound)
