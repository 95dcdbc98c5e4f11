"""Device-side helpers for the GPU tests (torch tensors as device buffers)."""
from __future__ import annotations

import ctypes as C

import numpy as np

import fdtd_gb300 as fg


def make_params(dims, consts, sources, jz, default=(0.0, 1.0, 1.0, 0.0)):
    """A FdtdParams for given constants; the arrays it points to are kept on it."""
    raw = fg.FdtdParams()
    raw.nx, raw.ny, raw.nz = dims
    for k in ("dt", "dx", "dy", "dz", "mu0", "eps0"):
        setattr(raw, k, consts[k])
    src = (C.c_int * max(1, 3 * len(sources)))(*[v for s in sources for v in s])
    raw.sourcesCount = len(sources)
    raw.sources = C.cast(src, C.POINTER(C.c_int))
    jz = np.ascontiguousarray(jz, np.float32)
    raw.jzCount = jz.size
    raw.jz = jz.ctypes.data_as(C.POINTER(C.c_float))
    raw.defaultSigma, raw.defaultEpsS, raw.defaultEpsI, raw.defaultTauD = default
    raw.waveFrequency = 1e9
    raw.pi = np.float32(np.pi)
    raw._keep = (src, jz)
    return raw


class Params:
    """Minimal stand-in for fg.Params that does not free caller memory."""

    def __init__(self, raw):
        self.raw = raw

    def __getattr__(self, k):
        return getattr(self.raw, k)

    @property
    def shape(self):
        return (self.raw.nz, self.raw.ny, self.raw.nx)


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def zeros(torch, shape):
    return torch.zeros(shape, dtype=torch.float32, device="cuda")


def ptr(t):
    return C.c_void_p(t.data_ptr())


class NativeState:
    """Device state of the native path: H x2, E x2, D x2, material."""

    def __init__(self, torch, shape, codes):
        self.h = [[zeros(torch, shape) for _ in range(3)] for _ in range(2)]
        self.e = [[zeros(torch, shape) for _ in range(3)] for _ in range(2)]
        self.d = [[zeros(torch, shape) for _ in range(3)] for _ in range(2)]
        self.mat = torch.from_numpy(np.ascontiguousarray(codes, np.uint8)).cuda()

    def fields(self, n: int, single_pass: bool) -> fg.NativeFields:
        cur, prv = (n + 1) % 2, n % 2
        hin, hout = (n % 2, (n + 1) % 2) if single_pass else (0, 0)
        f = fg.NativeFields()
        for k, c in enumerate("xyz"):
            setattr(f, "h" + c, self.h[hin][k].data_ptr())
            setattr(f, "h" + c + "_out", self.h[hout][k].data_ptr())
            setattr(f, "e" + c, self.e[cur][k].data_ptr())
            setattr(f, "e" + c + "_prev", self.e[prv][k].data_ptr())
            setattr(f, "d" + c, self.d[cur][k].data_ptr())
            setattr(f, "d" + c + "_prev", self.d[prv][k].data_ptr())
        f.material = self.mat.data_ptr()
        return f

    def latest(self, steps: int, single_pass: bool) -> dict[str, np.ndarray]:
        k = (steps - 1) % 2
        hk = steps % 2 if single_pass else 0
        out = {}
        for c, n in enumerate("xyz"):
            out["h" + n] = self.h[hk][c].cpu().numpy()
            out["e" + n] = self.e[k][c].cpu().numpy()
            out["d" + n] = self.d[k][c].cpu().numpy()
        return out


def run_native(torch, raw, specs, codes, rp, steps, scheme=fg.SCHEME_REFERENCE, mode="single"):
    """Runs `steps` native steps through fdtd_plan/fdtd_step(_h/_de)."""
    p = Params(raw)
    plan = fg.Plan(p, specs, scheme=scheme, rp=rp)
    st = NativeState(torch, p.shape, codes)
    L = fg.lib()
    single = mode == "single"
    for n in range(steps):
        f = st.fields(n, single)
        if single:
            fg.check(L.fdtd_step(plan.handle, C.byref(f), n, None), "fdtd_step")
        else:
            fg.check(L.fdtd_step_h(plan.handle, C.byref(f), None), "fdtd_step_h")
            fg.check(L.fdtd_step_de(plan.handle, C.byref(f), n, None), "fdtd_step_de")
    torch.cuda.synchronize()
    out = st.latest(steps, single)
    plan.close()
    return out
