"""fdtd_step_static: a single-pass step that allocates no device memory.

Callers that cannot call cudaMalloc (device memory owned by another
allocator, or a context where allocating is not allowed) use this entry
point; its per-class table, source sample and error word live in a static
device array.  The test calls it through the C ABI twice in a row and checks
each result against fdtd_step, which uses an allocated plan, starting from
the same random state.  This file is collected last on purpose.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import fdtd_gb300 as fg

from .gpu_util import NativeState, Params, dev, make_params
from .helpers import REL_L2_TOL, assert_fields_close, random_case

pytestmark = pytest.mark.gpu


def _random_state(torch, st: NativeState, rng):
    for group in (st.h, st.e, st.d):
        for slot in group:
            for t in slot:
                t.copy_(torch.from_numpy(rng.standard_normal(tuple(t.shape)).astype(np.float32)))


def _clone_state(torch, src: NativeState, dst: NativeState):
    for a, b in zip(src.h + src.e + src.d, dst.h + dst.e + dst.d):
        for x, y in zip(a, b):
            y.copy_(x)


@pytest.mark.parametrize("scheme", [fg.SCHEME_REFERENCE, fg.SCHEME_CORRECTED])
@pytest.mark.parametrize("dims", [(64, 24, 40), (37, 13, 11)])
def test_static_step_matches_planned_step_two_calls(cuda, dims, scheme):
    torch = cuda
    nx, ny, nz = dims
    codes, specs, rp, sources, consts, jz = random_case(nx, ny, nz, seed=31, ncls=7, nsrc=3)
    raw = make_params(dims, consts, sources, jz)
    p = Params(raw)
    plan = fg.Plan(p, specs, scheme=scheme, rp=rp)
    rng = np.random.default_rng(5)
    a = NativeState(torch, p.shape, codes)
    b = NativeState(torch, p.shape, codes)
    _random_state(torch, a, rng)
    _clone_state(torch, a, b)
    torch.cuda.synchronize()
    rp_dev = [dev(torch, r) for r in rp]
    rp_ptrs = (C.c_void_p * 6)(*[t.data_ptr() for t in rp_dev])
    L = fg.lib()
    for n in (0, 1):
        fa, fb = a.fields(n, True), b.fields(n, True)
        fg.check(L.fdtd_step(plan.handle, C.byref(fa), n, None), "fdtd_step")
        fg.check(L.fdtd_step_static(C.byref(raw), fg.fptr(np.ascontiguousarray(specs)), len(specs), scheme,
                                    C.byref(fb), rp_ptrs, n, None), "fdtd_step_static")
        torch.cuda.synchronize()
        assert_fields_close(b.latest(n + 1, True), a.latest(n + 1, True), tol=REL_L2_TOL)
    plan.close()


def test_static_step_rejects_too_many_classes(cuda):
    torch = cuda
    dims = (32, 8, 6)
    codes, specs, rp, sources, consts, jz = random_case(*dims, seed=2, ncls=5, nsrc=1)
    raw = make_params(dims, consts, sources, jz)
    st = NativeState(torch, (dims[2], dims[1], dims[0]), codes)
    big = np.zeros((fg.STATIC_MAX_CLASSES + 1, 4), np.float32)
    big[:, 1:3] = 1.0
    rp_dev = [dev(torch, r) for r in rp]
    rp_ptrs = (C.c_void_p * 6)(*[t.data_ptr() for t in rp_dev])
    f = st.fields(0, True)
    assert fg.lib().fdtd_step_static(C.byref(raw), fg.fptr(big), len(big), fg.SCHEME_REFERENCE, C.byref(f),
                                     rp_ptrs, 0, None) == fg.FDTD_ERR_INVALID


def test_static_step_requires_jz_table_with_sources(cuda):
    torch = cuda
    dims = (32, 8, 6)
    codes, specs, rp, sources, consts, jz = random_case(*dims, seed=3, ncls=4, nsrc=2)
    raw = make_params(dims, consts, sources, jz)
    raw.jz = None
    raw.jzCount = 0
    st = NativeState(torch, (dims[2], dims[1], dims[0]), codes)
    rp_dev = [dev(torch, r) for r in rp]
    rp_ptrs = (C.c_void_p * 6)(*[t.data_ptr() for t in rp_dev])
    f = st.fields(0, True)
    assert fg.lib().fdtd_step_static(C.byref(raw), fg.fptr(np.ascontiguousarray(specs)), len(specs),
                                     fg.SCHEME_CORRECTED, C.byref(f), rp_ptrs, 0, None) == fg.FDTD_ERR_INVALID


def test_static_step_source_sample_beyond_table_length(cuda):
    """A caller table longer than FDTD_JZ_LEN: the plan keeps its first
    FDTD_JZ_LEN samples, so beyond them both calls inject 0 (the large values
    planted past that length must not appear)."""
    torch = cuda
    dims = (40, 12, 10)
    codes, specs, rp, sources, consts, _ = random_case(*dims, seed=8, ncls=5, nsrc=2)
    jz = np.full(fg.JZ_LEN + 4096, 1e3, np.float32)
    jz[:fg.JZ_LEN] = np.random.default_rng(4).standard_normal(fg.JZ_LEN).astype(np.float32) * 1e-3
    raw = make_params(dims, consts, sources, jz)
    p = Params(raw)
    plan = fg.Plan(p, specs, scheme=fg.SCHEME_CORRECTED, rp=rp)
    rp_dev = [dev(torch, r) for r in rp]
    rp_ptrs = (C.c_void_p * 6)(*[t.data_ptr() for t in rp_dev])
    L = fg.lib()
    for n in (fg.JZ_LEN - 1, fg.JZ_LEN + 100):
        a = NativeState(torch, p.shape, codes)
        b = NativeState(torch, p.shape, codes)
        _random_state(torch, a, np.random.default_rng(n))
        _clone_state(torch, a, b)
        torch.cuda.synchronize()
        fa, fb = a.fields(n, True), b.fields(n, True)
        fg.check(L.fdtd_step(plan.handle, C.byref(fa), n, None), "fdtd_step")
        fg.check(L.fdtd_step_static(C.byref(raw), fg.fptr(np.ascontiguousarray(specs)), len(specs),
                                    fg.SCHEME_CORRECTED, C.byref(fb), rp_ptrs, n, None), "fdtd_step_static")
        torch.cuda.synchronize()
        assert_fields_close(b.latest(n + 1, True), a.latest(n + 1, True), tol=REL_L2_TOL)
    plan.close()
