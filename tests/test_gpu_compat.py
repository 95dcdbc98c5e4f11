"""Reference-compatible launchers (fdtd_update_*) against the reference's own
kernels (golden runs) and the FP32 oracle, through the C ABI."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import fdtd_gb300 as fg
from oracle import pyoracle as po

from .gpu_util import dev, make_params, ptr, zeros
from .helpers import REL_L2_TOL, RUNS, class_media, load_run, random_case, rel_l2

pytestmark = pytest.mark.gpu


def run_compat(torch, dims, consts, sources, jz, media, steps):
    """The reference main loop (fdtd.cu:115-530) driven through the compat ABI."""
    nx, ny, nz = dims
    shape = (nz, ny, nx)
    raw = make_params(dims, consts, sources, jz)
    L = fg.lib()
    fg.check(L.fdtd_copy_symbols(C.byref(raw)), "fdtd_copy_symbols")
    h = [zeros(torch, shape) for _ in range(3)]
    e = [[zeros(torch, shape) for _ in range(3)] for _ in range(3)]
    d = [[zeros(torch, shape) for _ in range(3)] for _ in range(3)]
    m = [dev(torch, a) for a in (media.sigma, media.eps_i, media.eps_s, media.tau_d)]
    rp = [dev(torch, r) for r in media.rp]
    P = lambda ts: [ptr(t) for t in ts]  # noqa: E731
    for i in range(steps):
        t, n0, n1 = i % 3, (i + 2) % 3, (i + 1) % 3
        fg.check(L.fdtd_update_h(*P(h), *P(e[n0]), None))
        fg.check(L.fdtd_update_d(*P(d[t]), *P(d[n0]), *P(h), None))
        fg.check(L.fdtd_update_sources(ptr(d[t][2]), ptr(d[n0][2]), ptr(h[0]), ptr(h[1]), i - i % 3, None))
        fg.check(L.fdtd_update_e(*P(e[t]), *P(e[n0]), *P(e[n1]), *P(d[t]), *P(d[n0]), *P(d[n1]), *P(m), None))
        fg.check(L.fdtd_update_mur(*P(e[t]), *P(e[n0]), *P(rp), None))
    torch.cuda.synchronize()
    return [a.cpu().numpy() for a in h + [x for s in e for x in s] + [x for s in d for x in s]]


@pytest.mark.parametrize("name", RUNS)
def test_compat_loop_matches_reference_run(cuda, name):
    g = load_run(name)
    got = run_compat(cuda, g.dims, g.consts, g.sources, g.jz, g.media, g.steps)
    for k, (a, b) in enumerate(zip(got, g.state)):
        assert rel_l2(a, b) <= REL_L2_TOL, f"array {k}: {rel_l2(a, b)}"


def test_each_compat_kernel_matches_oracle(cuda):
    """One call of each launcher on random inputs against the FP32 oracle."""
    torch = cuda
    nx, ny, nz = 37, 13, 9
    codes, specs, rp, sources, consts, jz = random_case(nx, ny, nz, seed=21, nsrc=3)
    media = class_media(codes, specs, rp)
    rng = np.random.default_rng(4)
    sh = (nz, ny, nx)
    rnd = lambda: rng.standard_normal(sh).astype(np.float32)  # noqa: E731
    cfg = po.make_cfg((nx, ny, nz), jz, sources=sources, consts=consts)
    raw = make_params((nx, ny, nz), consts, sources, jz)
    L = fg.lib()
    fg.check(L.fdtd_copy_symbols(C.byref(raw)))
    lib32 = po.lib("f32")
    Pf = C.POINTER(C.c_float)
    arr3 = lambda xs: (Pf * 3)(*[x.ctypes.data_as(Pf) for x in xs])  # noqa: E731

    # H
    h = [rnd() for _ in range(3)]
    e = [rnd() for _ in range(3)]
    hd = [dev(torch, a) for a in h]
    ed = [dev(torch, a) for a in e]  # keep every device buffer referenced until the launch completes
    fg.check(L.fdtd_update_h(*[ptr(t) for t in hd], *[ptr(t) for t in ed], None))
    lib32.oracle_update_h(C.byref(cfg), arr3(h), arr3(e))
    torch.cuda.synchronize()
    for a, b in zip(hd, h):
        assert rel_l2(a.cpu().numpy(), b) < 1e-6

    # D and sources
    dT = [np.zeros(sh, np.float32) for _ in range(3)]
    dS = [rnd() for _ in range(3)]
    dTd = [zeros(torch, sh) for _ in range(3)]
    hdv = [dev(torch, a) for a in h]
    dSd = [dev(torch, a) for a in dS]
    fg.check(L.fdtd_update_d(*[ptr(t) for t in dTd], *[ptr(t) for t in dSd], *[ptr(t) for t in hdv], None))
    fg.check(L.fdtd_update_sources(ptr(dTd[2]), ptr(dSd[2]), ptr(hdv[0]), ptr(hdv[1]), 6, None))
    lib32.oracle_update_d(C.byref(cfg), arr3(dT), arr3(dS), arr3(h), 6)
    torch.cuda.synchronize()
    for a, b in zip(dTd, dT):
        assert rel_l2(a.cpu().numpy(), b) < 1e-6

    # E
    eT = [np.zeros(sh, np.float32) for _ in range(3)]
    srcs = [[rnd() for _ in range(3)] for _ in range(5)]
    eTd = [zeros(torch, sh) for _ in range(3)]
    md = [dev(torch, a) for a in (media.sigma, media.eps_i, media.eps_s, media.tau_d)]
    srcd = [dev(torch, a) for s in srcs for a in s]
    fg.check(L.fdtd_update_e(*[ptr(t) for t in eTd], *[ptr(t) for t in srcd], *[ptr(t) for t in md], None))
    ms = media.as_struct()
    lib32.oracle_update_e(C.byref(cfg), C.byref(ms), arr3(eT), *[arr3(s) for s in srcs])
    torch.cuda.synchronize()
    for a, b in zip(eTd, eT):
        assert rel_l2(a.cpu().numpy(), b) < 2e-6

    # Mur
    eS = [rnd() for _ in range(3)]
    eT2 = [rnd() for _ in range(3)]
    eT2d = [dev(torch, a) for a in eT2]
    rpd = [dev(torch, r) for r in rp]
    eSd = [dev(torch, a) for a in eS]
    fg.check(L.fdtd_update_mur(*[ptr(t) for t in eT2d], *[ptr(t) for t in eSd], *[ptr(t) for t in rpd], None))
    lib32.oracle_update_mur(C.byref(cfg), C.byref(ms), arr3(eT2), arr3(eS))
    torch.cuda.synchronize()
    for a, b in zip(eT2d, eT2):
        assert rel_l2(a.cpu().numpy(), b) < 1e-6


def test_compat_requires_symbols_on_device(cuda):
    # symbols were copied by earlier tests in this process or not; either the
    # call succeeds or reports FDTD_ERR_NO_SYMBOLS, never crashes
    raw = make_params((5, 5, 5), dict(dt=1e-12, dx=1e-3, dy=1e-3, dz=1e-3, mu0=1.2566371e-06, eps0=8.841941e-12),
                      [(0, 2, 2)], np.zeros(4, np.float32))
    assert fg.lib().fdtd_copy_symbols(C.byref(raw)) == fg.FDTD_ERR_INVALID  # source at x = 0
