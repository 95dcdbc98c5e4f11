"""Overlap of a step's single-pass kernel with the previous step's Mur kernel
(programmatic dependent launch inside the step graphs).  CTAs clear of the
faces start early; all others wait.  On a grid large enough to have such CTAs,
with sources both near faces and in the interior, the fields must equal, bit
for bit, a run of the same solver with the overlap off (a probe installed
puts the monitor kernel between Mur and the next step), and the FP64 oracle
within the FP32 tolerance."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from oracle import pyoracle as po

from .gpu_util import Params, make_params
from .helpers import assert_fields_close, class_media, random_case

pytestmark = pytest.mark.gpu

DIMS = (160, 48, 140)  # 5 x 6 tiles; 3 z chunks (D form) or 9 (compact form): inner CTAs exist


@pytest.mark.parametrize("kernel", [fg.KERNEL_SINGLE_PASS, fg.KERNEL_COMPACT])
def test_overlapped_steps_equal_serial_steps_and_oracle(cuda, kernel):
    steps = 90
    codes, specs, rp, _, consts, jz = random_case(*DIMS, seed=21, ncls=4, nsrc=0)
    sources = [(80, 24, 70), (3, 2, 1), (158, 46, 138), (100, 30, 50)]  # interior, corner, corner, interior
    raw = make_params(DIMS, consts, sources, jz)
    runs = {}
    for overlap in (True, False):
        with fg.Solver(Params(raw), codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel) as s:
            if not overlap:
                s.set_probes([(1, 1, 1)], capacity=steps)
            for chunk in (7, 40, 43):
                s.run(chunk)
            runs[overlap] = s.fields()
    for name in runs[True]:
        assert np.array_equal(runs[True][name].view(np.uint32), runs[False][name].view(np.uint32)), name
    p = po.OracleParams()
    p.nx, p.ny, p.nz = DIMS
    p.pi, p.wave_frequency, p.eps0 = raw.pi, raw.waveFrequency, raw.eps0
    p.default_sigma, p.default_eps_s = raw.defaultSigma, raw.defaultEpsS
    p.default_eps_i, p.default_tau_d = raw.defaultEpsI, raw.defaultTauD
    media = class_media(codes, specs, po.uniform_media(p).rp)
    st = po.State(*DIMS, np.float64)
    po.run(po.make_cfg(DIMS, jz, sources=sources, consts=consts, corrected=True), media, st, 0, steps)
    want = st.latest(steps)
    assert_fields_close(runs[True], want, names=[n for n in runs[True]])


@pytest.mark.parametrize("kernel", [fg.KERNEL_SINGLE_PASS, fg.KERNEL_COMPACT])
def test_sources_on_z_chunk_borders(cuda, kernel):
    """Sources on the planes where z chunks meet: the last plane of a chunk
    (which the next chunk also stages, to recompute H below its first plane),
    the first plane of the next chunk, and a pair on the planes either side of
    a border; against the FP64 oracle."""
    dims = (70, 26, 150)
    # nz is split into equal chunks of at most 64 planes (D form: 3 of 50) or
    # at most 16 (compact form: 10 of 15)
    zc = 50 if kernel == fg.KERNEL_SINGLE_PASS else 15
    steps = 60
    codes, specs, rp, _, consts, jz = random_case(*dims, seed=5, ncls=3, nsrc=0)
    sources = [(35, 13, zc - 1), (20, 7, zc), (50, 20, 2 * zc - 1), (40, 10, 2 * zc), (41, 11, 2 * zc + 1)]
    raw = make_params(dims, consts, sources, jz)
    with fg.Solver(Params(raw), codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel) as s:
        s.run(steps)
        got = s.fields()
    p = po.OracleParams()
    p.nx, p.ny, p.nz = dims
    p.pi, p.wave_frequency, p.eps0 = raw.pi, raw.waveFrequency, raw.eps0
    p.default_sigma, p.default_eps_s = raw.defaultSigma, raw.defaultEpsS
    p.default_eps_i, p.default_tau_d = raw.defaultEpsI, raw.defaultTauD
    media = class_media(codes, specs, po.uniform_media(p).rp)
    st = po.State(*dims, np.float64)
    po.run(po.make_cfg(dims, jz, sources=sources, consts=consts, corrected=True), media, st, 0, steps)
    assert_fields_close(got, st.latest(steps), names=list(got))
