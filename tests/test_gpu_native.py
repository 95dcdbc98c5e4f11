"""Native fused path (fdtd_step, fdtd_step_h + fdtd_step_de) through the C ABI
against the reference's golden runs and the oracle."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from oracle import pyoracle as po

from .gpu_util import make_params, run_native
from .helpers import REL_L2_TOL, assert_fields_close, class_media, load_run, random_case

pytestmark = pytest.mark.gpu

CLASS_RUNS = ["sphere24", "classes70x20x9"]


@pytest.mark.parametrize("mode", ["single", "two_pass"])
@pytest.mark.parametrize("name", CLASS_RUNS)
def test_native_matches_reference_run(cuda, name, mode):
    g = load_run(name)
    raw = make_params(g.dims, g.consts, g.sources, g.jz)
    got = run_native(cuda, raw, g.specs, g.codes, g.media.rp, g.steps, mode=mode)
    assert_fields_close(got, g.latest())


@pytest.mark.parametrize("mode", ["single", "two_pass"])
@pytest.mark.parametrize("dims,seed", [((33, 17, 12), 1), ((64, 9, 7), 2), ((5, 40, 6), 3), ((129, 3, 4), 4)])
def test_native_matches_fp32_oracle_reference_scheme(cuda, dims, seed, mode):
    nx, ny, nz = dims
    codes, specs, rp, sources, consts, jz = random_case(nx, ny, nz, seed, nsrc=3)
    steps = 14
    media = class_media(codes, specs, rp)
    st = po.State(nx, ny, nz, np.float32)
    po.run(po.make_cfg(dims, jz, sources=sources, consts=consts), media, st, 0, steps)
    want = st.latest(steps)
    raw = make_params(dims, consts, sources, jz)
    got = run_native(cuda, raw, specs, codes, rp, steps, mode=mode)
    assert_fields_close(got, want)


@pytest.mark.parametrize("mode", ["single", "two_pass"])
def test_native_mixed_one_valued_and_varying_mur_slabs(cuda, mode):
    """A slab whose entries are all one value takes the Mur kernel's
    constant-factor path (and, for an x slab, a factor table filled on the
    device), any other slab the slab path: three of each, against the FP32
    oracle on the same slabs."""
    dims = (40, 24, 18)
    nx, ny, nz = dims
    codes, specs, rp, sources, consts, jz = random_case(nx, ny, nz, 11, nsrc=2)
    for k in (0, 2, 4):  # x = 0, z = 0 and y = ny-1 slabs one-valued
        rp[k] = np.full_like(rp[k], rp[k].flat[0])
    steps = 14
    media = class_media(codes, specs, rp)
    st = po.State(nx, ny, nz, np.float32)
    po.run(po.make_cfg(dims, jz, sources=sources, consts=consts), media, st, 0, steps)
    want = st.latest(steps)
    raw = make_params(dims, consts, sources, jz)
    got = run_native(cuda, raw, specs, codes, rp, steps, mode=mode)
    assert_fields_close(got, want)


@pytest.mark.parametrize("mode", ["single", "two_pass"])
def test_native_corrected_scheme_matches_fp64_oracle(cuda, mode):
    dims = (41, 23, 19)
    nx, ny, nz = dims
    codes, specs, rp, sources, consts, jz = random_case(nx, ny, nz, 7, nsrc=2)
    steps = 60
    media = class_media(codes, specs, rp)
    st = po.State(nx, ny, nz, np.float64)
    po.run(po.make_cfg(dims, jz, sources=sources, consts=consts, corrected=True), media, st, 0, steps)
    want = st.latest(steps)
    raw = make_params(dims, consts, sources, jz)
    got = run_native(cuda, raw, specs, codes, rp, steps, scheme=fg.SCHEME_CORRECTED, mode=mode)
    assert_fields_close(got, want, tol=REL_L2_TOL)


def test_single_pass_rejects_in_place_h(cuda):
    import ctypes as C

    from .gpu_util import NativeState, Params

    g = load_run("sphere24")
    raw = make_params(g.dims, g.consts, g.sources, g.jz)
    plan = fg.Plan(Params(raw), g.specs, rp=g.media.rp)
    st = NativeState(cuda, Params(raw).shape, g.codes)
    f = st.fields(0, single_pass=False)  # H in place
    assert fg.lib().fdtd_step(plan.handle, C.byref(f), 0, None) == fg.FDTD_ERR_INVALID
    plan.close()


@pytest.mark.parametrize("dims,seed", [((48, 20, 70), 5), ((32, 8, 130), 6), ((64, 64, 64), 8), ((96, 7, 9), 9)])
def test_single_pass_tma_path_and_chunk_borders(cuda, dims, seed):
    """nx a multiple of 16 selects the TMA staging; nz > 64 splits z into
    chunks whose first plane recomputes H of the plane below."""
    nx, ny, nz = dims
    codes, specs, rp, sources, consts, jz = random_case(nx, ny, nz, seed, nsrc=4)
    steps = 9
    media = class_media(codes, specs, rp)
    st = po.State(nx, ny, nz, np.float32)
    po.run(po.make_cfg(dims, jz, sources=sources, consts=consts), media, st, 0, steps)
    raw = make_params(dims, consts, sources, jz)
    got = run_native(cuda, raw, specs, codes, rp, steps, mode="single")
    assert_fields_close(got, st.latest(steps))


@pytest.mark.parametrize("chunk", [1, 2, 5])
@pytest.mark.parametrize("dims", [(32, 16, 23), (37, 11, 17)])
def test_single_pass_small_z_chunks(cuda, monkeypatch, dims, chunk):
    monkeypatch.setenv("FDTD_ZCHUNK", str(chunk))
    nx, ny, nz = dims
    codes, specs, rp, sources, consts, jz = random_case(nx, ny, nz, 10 + chunk, nsrc=3)
    steps = 8
    media = class_media(codes, specs, rp)
    st = po.State(nx, ny, nz, np.float32)
    po.run(po.make_cfg(dims, jz, sources=sources, consts=consts), media, st, 0, steps)
    raw = make_params(dims, consts, sources, jz)
    got = run_native(cuda, raw, specs, codes, rp, steps, mode="single")
    assert_fields_close(got, st.latest(steps))


@pytest.mark.parametrize("dims,seed", [((64, 40, 70), 12), ((48, 17, 9), 13), ((33, 26, 10), 14)])
def test_single_pass_both_schemes(cuda, dims, seed):
    """Single-pass kernel in both schemes (TMA staging for nx % 16 == 0,
    cp.async otherwise) against the FP32 / FP64 oracle."""
    nx, ny, nz = dims
    codes, specs, rp, sources, consts, jz = random_case(nx, ny, nz, seed, nsrc=3)
    steps = 7
    media = class_media(codes, specs, rp)
    for corrected in (False, True):
        st = po.State(nx, ny, nz, np.float32 if not corrected else np.float64)
        po.run(po.make_cfg(dims, jz, sources=sources, consts=consts, corrected=corrected), media, st, 0, steps)
        raw = make_params(dims, consts, sources, jz)
        got = run_native(cuda, raw, specs, codes, rp, steps, mode="single",
                         scheme=fg.SCHEME_CORRECTED if corrected else fg.SCHEME_REFERENCE)
        assert_fields_close(got, st.latest(steps))
