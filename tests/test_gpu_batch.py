"""Batched solves (fdtd_batch_*): every solve of a mixed batch equals the same
solve run alone and the oracle, including solves added while others run."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from oracle import pyoracle as po

from .gpu_util import Params, make_params
from .helpers import assert_fields_close, class_media, random_case

pytestmark = pytest.mark.gpu

CASES = [  # dims, steps, scheme
    ((48, 37, 29), 30, fg.SCHEME_REFERENCE),
    ((64, 64, 40), 45, fg.SCHEME_CORRECTED),
    ((33, 50, 70), 20, fg.SCHEME_REFERENCE),
    ((96, 20, 16), 60, fg.SCHEME_CORRECTED),
    ((17, 9, 11), 12, fg.SCHEME_REFERENCE),
]


def _case(k):
    dims, steps, scheme = CASES[k]
    codes, specs, rp, sources, consts, jz = random_case(*dims, seed=100 + k, ncls=4, nsrc=2)
    raw = make_params(dims, consts, sources, jz, default=(0.0, 1.0, 1.0, 0.0))
    return dims, steps, scheme, codes, specs, sources, consts, jz, raw


def _oracle(dims, steps, scheme, codes, specs, sources, consts, jz, raw):
    p = po.OracleParams()
    p.nx, p.ny, p.nz = dims
    p.pi, p.wave_frequency, p.eps0 = raw.pi, raw.waveFrequency, raw.eps0
    p.default_sigma, p.default_eps_s = raw.defaultSigma, raw.defaultEpsS
    p.default_eps_i, p.default_tau_d = raw.defaultEpsI, raw.defaultTauD
    media = class_media(codes, specs, po.uniform_media(p).rp)
    corrected = scheme == fg.SCHEME_CORRECTED
    st = po.State(*dims, np.float64 if corrected else np.float32)
    po.run(po.make_cfg(dims, jz, sources=sources, consts=consts, corrected=corrected), media, st, 0, steps)
    return st.latest(steps)


def test_mixed_batch_matches_lone_solves_and_oracle(cuda):
    b = fg.Batch()
    ids = []
    cases = [_case(k) for k in range(len(CASES))]
    for dims, steps, scheme, codes, specs, sources, consts, jz, raw in cases:
        ids.append(b.add(Params(raw), codes, specs, steps, scheme=scheme))
    assert len(b) == len(CASES)
    b.run(max(c[1] for c in cases) + 5)  # every solve stops at its own target
    for sid, case in zip(ids, cases):
        dims, steps, scheme, codes, specs, sources, consts, jz, raw = case
        assert b.steps(sid) == steps
        got = b.fields(sid)
        # alone: the single-solve path on the same inputs
        with fg.Solver(Params(raw), codes, specs, scheme=scheme) as s:
            s.run(steps)
            alone = s.fields()
        for name in got:
            assert np.array_equal(got[name].view(np.uint32), alone[name].view(np.uint32)), (dims, name)
        assert_fields_close(got, _oracle(*case))
    b.close()


def test_solves_added_and_removed_while_running(cuda):
    b = fg.Batch()
    c0, c1, c2 = _case(0), _case(1), _case(3)
    i0 = b.add(Params(c0[8]), c0[3], c0[4], c0[1], scheme=c0[2])
    i1 = b.add(Params(c1[8]), c1[3], c1[4], c1[1], scheme=c1[2])
    b.run(10)
    i2 = b.add(Params(c2[8]), c2[3], c2[4], c2[1], scheme=c2[2])
    b.run(15)
    b.remove(i0)  # finished or not, its memory is released
    b.run(60)
    assert b.steps(i1) == c1[1] and b.steps(i2) == c2[1]
    for sid, case in ((i1, c1), (i2, c2)):
        assert_fields_close(b.fields(sid), _oracle(*case))
    b.close()


def test_solve_bytes_accounts_state():
    assert fg.Batch.solve_bytes(64, 64, 64) >= 73 * 64 ** 3
    assert fg.Batch.solve_bytes(2, 64, 64) == 0


def test_compact_batch_matches_lone_compact_solves_and_oracle(cuda):
    """A batch of the compact form: every solve equals the compact solver run
    alone bit for bit and the oracle within the FP32 tolerance (E, H); D is
    not readable."""
    b = fg.Batch(kernel=fg.KERNEL_COMPACT)
    cases = [_case(k) for k in range(len(CASES))]
    ids = [b.add(Params(c[8]), c[3], c[4], c[1], scheme=c[2]) for c in cases]
    assert b.need_bytes(64, 64, 64) < fg.Batch.solve_bytes(64, 64, 64)
    b.run(max(c[1] for c in cases) + 3)
    for sid, case in zip(ids, cases):
        dims, steps, scheme, codes, specs, sources, consts, jz, raw = case
        assert b.steps(sid) == steps
        got = b.fields(sid)
        assert sorted(got) == ["ex", "ey", "ez", "hx", "hy", "hz"]
        with pytest.raises(fg.FdtdError):
            b.field(sid, "dz")
        with fg.Solver(Params(raw), codes, specs, scheme=scheme, kernel=fg.KERNEL_COMPACT) as s:
            s.run(steps)
            alone = s.fields()
        for name in got:
            assert np.array_equal(got[name].view(np.uint32), alone[name].view(np.uint32)), (dims, name)
        assert_fields_close(got, _oracle(*case), names=list(got))
    b.close()


def test_compact16_batch_matches_lone_solves_and_oracle(cuda):
    """A batch of the 16-bit-R compact form: every solve equals the same form
    run alone bit for bit (the batch pads rows to 16 cells and stages R by
    TMA; alone, rows that are not a multiple of 16 read R directly) and the
    oracle within the reduced-storage tolerance; it needs less memory than the
    32-bit compact form."""
    b = fg.Batch(kernel=fg.KERNEL_COMPACT_R16)
    b32 = fg.Batch(kernel=fg.KERNEL_COMPACT)
    assert b.need_bytes(64, 64, 64) < b32.need_bytes(64, 64, 64)
    b32.close()
    cases = [_case(k) for k in range(len(CASES))]
    ids = [b.add(Params(c[8]), c[3], c[4], c[1], scheme=c[2]) for c in cases]
    b.run(max(c[1] for c in cases) + 3)
    for sid, case in zip(ids, cases):
        dims, steps, scheme, codes, specs, sources, consts, jz, raw = case
        assert b.steps(sid) == steps
        got = b.fields(sid)
        assert sorted(got) == ["ex", "ey", "ez", "hx", "hy", "hz"]
        with fg.Solver(Params(raw), codes, specs, scheme=scheme, kernel=fg.KERNEL_COMPACT_R16) as s:
            s.run(steps)
            alone = s.fields()
        for name in got:
            assert np.array_equal(got[name].view(np.uint32), alone[name].view(np.uint32)), (dims, name)
        assert_fields_close(got, _oracle(*case), tol=1e-3, names=list(got))
    b.close()


@pytest.mark.parametrize("kernel", [fg.KERNEL_SINGLE_PASS, fg.KERNEL_COMPACT, fg.KERNEL_COMPACT_R16])
def test_autotuned_batch_gives_the_same_bits(cuda, kernel):
    """fdtd_batch_autotune times real steps of the solves at each candidate
    (compact forms: the four strip tile shapes and the z-marching kernel, each
    with four z-chunk limits; D form: five z-chunk limits) and keeps the
    fastest.  A cell's update depends neither on where tiles and chunks meet
    nor on the kernel, so every solve still equals the same solve run alone,
    bit for bit, and the steps taken while tuning count."""
    compact = kernel in fg.COMPACT_KERNELS
    cands, trials = ((8, 16, 32, 64), 20) if compact else ((16, 24, 32, 48, 64), 5)
    steps = 16 * trials + 80  # outlasts the trials (16 steps each)
    b = fg.Batch(kernel=kernel)
    cases = [_case(k) for k in range(len(CASES))]
    ids = [b.add(Params(c[8]), c[3], c[4], steps, scheme=c[2]) for c in cases]
    chosen = b.autotune(steps_per_trial=8)
    assert chosen in cands
    t = b.tuning()
    assert t["z_chunk_limit"] == chosen
    if compact:
        assert t["strip_shape"] in (-1, 0, 1, 2, 3) and t["tile_rows"] in (8, 16), t
    done = b.steps(ids[0])
    assert 16 * trials - 8 <= done <= 16 * trials, done
    b.run(steps - done)
    for sid, case in zip(ids, cases):
        dims, _, scheme, codes, specs, sources, consts, jz, raw = case
        assert b.steps(sid) == steps
        got = b.fields(sid)
        with fg.Solver(Params(raw), codes, specs, scheme=scheme, kernel=kernel) as s:
            s.run(steps)
            alone = s.fields()
        for name in got:
            assert np.array_equal(got[name].view(np.uint32), alone[name].view(np.uint32)), (dims, name)
    b.close()
