"""ctypes binding of the oracle libraries (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker or as the timed CPU baseline.  Nothing in the
``fdtd_gb300`` package imports it.

State layout follows the reference (fdtd.h:37-54): H, three E slots, three D
slots, each a C-contiguous (nz, ny, nx) array, x fastest.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import build as _build

JZ_LEN = 1 << 16
SPEC_CODES = 256


class OracleParams(C.Structure):
    """Mirror of ``oracle_params`` (and of ``ref_flat_params``)."""

    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("iterations", C.c_int),
        ("input_path", C.c_char * 1024), ("output_path", C.c_char * 1024),
        ("elements_per_wave", C.c_int), ("wave_frequency", C.c_float), ("pulse_width", C.c_float),
        ("pulse_modulation_frequency", C.c_float), ("nsources", C.c_int), ("sources", C.c_int * 192),
        ("default_sigma", C.c_float), ("default_eps_s", C.c_float), ("default_eps_i", C.c_float),
        ("default_tau_d", C.c_float),
        ("pi", C.c_float), ("c", C.c_float), ("timeskip", C.c_float), ("lambda_", C.c_float),
        ("dt", C.c_float), ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float),
        ("mu0", C.c_float), ("eps0", C.c_float),
    ]

    def source_list(self) -> list[tuple[int, int, int]]:
        return [tuple(self.sources[3 * k:3 * k + 3]) for k in range(self.nsources)]


class OracleCfg(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dt", C.c_float), ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float),
        ("mu0", C.c_float), ("eps0", C.c_float),
        ("nsources", C.c_int), ("sources", C.POINTER(C.c_int)),
        ("jz", C.POINTER(C.c_float)), ("njz", C.c_int),
        ("corrected", C.c_int), ("nthreads", C.c_int),
    ]


class OracleMedia(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_float)) for n in
                ("sigma", "eps_i", "eps_s", "tau_d", "rpx0", "rpy0", "rpz0", "rpx_end", "rpy_end", "rpz_end")]


def _ptr(a: np.ndarray, ctype=C.c_float):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(ctype))


_LIBS: dict[str, C.CDLL] = {}


def lib(tag: str) -> C.CDLL:
    """Load ``f64``, ``f32``, ``ref_cpu`` or ``ref_host`` (building on demand)."""
    if tag not in _LIBS:
        if tag in ("f64", "f32"):
            path = _build.build_oracle()[tag]
        else:
            libs = _build.build_reference()
            if libs is None:
                raise FileNotFoundError("reference sources are not present on this machine")
            path = libs["cpu" if tag == "ref_cpu" else "host"]
        _LIBS[tag] = C.CDLL(str(path))
    return _LIBS[tag]


# ----------------------------------------------------------------- set-up

def params_read(path: str | Path, which: str = "f64") -> OracleParams:
    p = OracleParams()
    if which == "ref":
        rc = lib("ref_host").ref_host_params_read(str(path).encode(), C.byref(p))
    else:
        rc = lib(which).oracle_params_read(str(path).encode(), C.byref(p))
    if rc != 0:
        raise ValueError(f"params_read({path}) failed: {rc}")
    return p


def set_timeskip(p: OracleParams, timeskip: float, which: str = "f64") -> None:
    """dt for the Courant factor ``timeskip`` (the reference fixes 1.0)."""
    if lib(which).oracle_params_set_timeskip(C.byref(p), C.c_float(timeskip)) != 0:
        raise ValueError(f"set_timeskip({timeskip}) failed")


def read_specs(path, which: str = "f64") -> np.ndarray:
    """The mat_specs records as loadMaterials reads them: (256, 4) float32
    rows (sigma, eps_s, eps_i, tau) indexed by class code."""
    specs = np.zeros((SPEC_CODES, 4), np.float32)
    rc = lib(which).oracle_read_specs(str(path).encode(), _ptr(specs))
    if rc != 0:
        raise ValueError(f"read_specs({path}) failed: {rc}")
    return specs


def threads(cfg: "OracleCfg", which: str = "f64") -> int:
    """Host threads the oracle's loops run on for cfg."""
    return int(lib(which).oracle_threads(C.byref(cfg)))


def setup_sources(p: OracleParams, which: str = "f64") -> np.ndarray:
    jz = np.zeros(JZ_LEN, np.float32)
    if which == "ref":
        lib("ref_host").ref_host_setup_sources(C.byref(p), _ptr(jz))
    else:
        rc = lib(which).oracle_setup_sources(C.byref(p), _ptr(jz))
        if rc != 0:
            raise ValueError(f"setup_sources failed: {rc}")
    return jz


@dataclass
class Media:
    """Per-cell float material arrays and the six Mur rp slabs."""

    sigma: np.ndarray
    eps_i: np.ndarray
    eps_s: np.ndarray
    tau_d: np.ndarray
    rp: list[np.ndarray] = field(default_factory=list)  # x0, y0, z0, xEnd, yEnd, zEnd

    def as_struct(self) -> OracleMedia:
        m = OracleMedia()
        for name in ("sigma", "eps_i", "eps_s", "tau_d"):
            setattr(m, name, _ptr(getattr(self, name)))
        for name, arr in zip(("rpx0", "rpy0", "rpz0", "rpx_end", "rpy_end", "rpz_end"), self.rp):
            setattr(m, name, _ptr(arr))
        return m


def rp_shapes(nx: int, ny: int, nz: int) -> list[tuple[int, ...]]:
    return [(nz, ny, 2), (nz, 2, nx), (2, ny, nx)] * 2


def setup_mur(p: OracleParams, sigma, eps_s, eps_i, tau) -> list[np.ndarray]:
    rp = [np.zeros(s, np.float32) for s in rp_shapes(p.nx, p.ny, p.nz)]
    lib("f64").oracle_setup_mur(C.byref(p), _ptr(sigma), _ptr(eps_s), _ptr(eps_i), _ptr(tau),
                                *[_ptr(r) for r in rp])
    return rp


def uniform_media(p: OracleParams) -> Media:
    """Material arrays filled with the params' default material, as
    initFieldWithParams does (fdtd.cu:708-713), with Mur slabs from them."""
    shape = (p.nz, p.ny, p.nx)
    m = Media(sigma=np.full(shape, p.default_sigma, np.float32), eps_i=np.full(shape, p.default_eps_i, np.float32),
              eps_s=np.full(shape, p.default_eps_s, np.float32), tau_d=np.full(shape, p.default_tau_d, np.float32))
    m.rp = setup_mur(p, m.sigma, m.eps_s, m.eps_i, m.tau_d)
    return m


def load_materials(p: OracleParams, specs_path, pgm_dir, which: str = "f64", media: Media | None = None):
    """Returns (codes uint8 or None, specs (256,4) or None, sigma, eps_s, eps_i, tau)."""
    shape = (p.nz, p.ny, p.nx)
    arrs = [np.zeros(shape, np.float32) for _ in range(4)]
    if which == "ref":
        lib("ref_host").ref_host_load_materials(C.byref(p), str(specs_path).encode(), str(pgm_dir).encode(),
                                                *[_ptr(a) for a in arrs])
        return (None, None, *arrs)
    codes = np.zeros(shape, np.uint8)
    specs = np.zeros((SPEC_CODES, 4), np.float32)
    rc = lib(which).oracle_load_materials(C.byref(p), str(specs_path).encode(), str(pgm_dir).encode(), _ptr(specs),
                                          _ptr(codes, C.c_uint8), *[_ptr(a) for a in arrs])
    if rc != 0:
        raise ValueError(f"load_materials failed: {rc}")
    return (codes, specs, *arrs)


def write_snapshot3d(out_dir, fields9, iteration: int, which: str = "f64", p: OracleParams | None = None) -> None:
    nz, ny, nx = fields9[0].shape
    arr = (C.POINTER(C.c_float) * 9)(*[_ptr(np.ascontiguousarray(f, np.float32)) for f in fields9])
    if which == "ref":
        assert p is not None
        q = OracleParams()
        C.memmove(C.byref(q), C.byref(p), C.sizeof(OracleParams))
        q.output_path = str(out_dir).encode()
        q.nx, q.ny, q.nz = nx, ny, nz
        lib("ref_host").ref_host_write_snapshot3d(C.byref(q), arr, iteration)
    else:
        rc = lib("f64").oracle_write_snapshot3d(str(out_dir).encode(), nx, ny, nz, arr, iteration)
        if rc != 0:
            raise OSError(f"write_snapshot3d failed: {rc}")


# ------------------------------------------------------------- time loop

class State:
    """Reference state: 21 arrays (H, E slots 0-2, D slots 0-2)."""

    def __init__(self, nx: int, ny: int, nz: int, dtype=np.float64):
        self.shape = (nz, ny, nx)
        self.dtype = np.dtype(dtype)
        self.h = [np.zeros(self.shape, dtype) for _ in range(3)]
        self.e = [[np.zeros(self.shape, dtype) for _ in range(3)] for _ in range(3)]
        self.d = [[np.zeros(self.shape, dtype) for _ in range(3)] for _ in range(3)]

    def arrays(self) -> list[np.ndarray]:
        return self.h + [a for s in self.e for a in s] + [a for s in self.d for a in s]

    def latest(self, step_count: int) -> dict[str, np.ndarray]:
        """Fields after ``step_count`` steps from zero: E and D from the slot
        written last ((n-1) % 3), and H."""
        k = (step_count - 1) % 3
        out = {"hx": self.h[0], "hy": self.h[1], "hz": self.h[2]}
        for c, n in enumerate("xyz"):
            out["e" + n] = self.e[k][c]
            out["d" + n] = self.d[k][c]
        return out

    def previous(self, step_count: int) -> dict[str, np.ndarray]:
        """E and D one step older than ``latest``."""
        k = (step_count - 2) % 3
        out = {}
        for c, n in enumerate("xyz"):
            out["e" + n] = self.e[k][c]
            out["d" + n] = self.d[k][c]
        return out


def make_cfg(p_or_dims, jz: np.ndarray, sources=None, corrected: bool = False, nthreads: int = 0,
             consts: dict | None = None):
    """Build an OracleCfg (keeps references to the arrays it points at)."""
    if isinstance(p_or_dims, OracleParams):
        p = p_or_dims
        dims = (p.nx, p.ny, p.nz)
        consts = dict(dt=p.dt, dx=p.dx, dy=p.dy, dz=p.dz, mu0=p.mu0, eps0=p.eps0)
        if sources is None:
            sources = p.source_list()
    else:
        dims = p_or_dims
    src = np.ascontiguousarray(np.array(sources or [], np.int32).reshape(-1))
    jz = np.ascontiguousarray(jz, np.float32)
    cfg = OracleCfg(nx=dims[0], ny=dims[1], nz=dims[2], nsources=len(src) // 3, sources=_ptr(src, C.c_int),
                    jz=_ptr(jz), njz=len(jz), corrected=int(corrected), nthreads=nthreads, **consts)
    cfg._keep = (src, jz)
    return cfg


def run(cfg: OracleCfg, media: Media, state: State, step0: int, nsteps: int) -> None:
    tag = {8: "f64", 4: "f32"}[state.dtype.itemsize]
    ms = media.as_struct()
    st = state.arrays()
    ctype = C.c_double if tag == "f64" else C.c_float
    ptrs = [_ptr(a, ctype) for a in st]

    class S(C.Structure):
        _fields_ = [("p", C.POINTER(ctype) * 21)]

    s = S()
    for i, q in enumerate(ptrs):
        s.p[i] = q
    rc = lib(tag).oracle_run(C.byref(cfg), C.byref(ms), C.byref(s), step0, nsteps)
    if rc != 0:
        raise ValueError(f"oracle_run failed: {rc}")


def ref_cpu_run(cfg: OracleCfg, media: Media, state: State, step0: int, nsteps: int, nthreads: int = 0) -> None:
    """Run the reference's own kernels on the CPU (float32 state)."""
    assert state.dtype == np.float32
    L = lib("ref_cpu")
    src = cfg._keep[0]
    jz = cfg._keep[1]
    L.ref_cpu_set_symbols(cfg.nx, cfg.ny, cfg.nz, C.c_float(cfg.dt), C.c_float(cfg.dx), C.c_float(cfg.dy),
                          C.c_float(cfg.dz), C.c_float(cfg.mu0), C.c_float(cfg.eps0), cfg.nsources,
                          _ptr(src, C.c_int), _ptr(jz), len(jz))
    if nthreads > 0:
        L.ref_cpu_set_threads(nthreads)
    P = C.POINTER(C.c_float)
    st = (P * 21)(*[_ptr(a) for a in state.arrays()])
    m = (P * 4)(*[_ptr(a) for a in (media.sigma, media.eps_i, media.eps_s, media.tau_d)])
    rp = (P * 6)(*[_ptr(a) for a in media.rp])
    L.ref_cpu_run(st, m, rp, step0, nsteps)


# ------------------------------------------------- reference kernels on GPU

class RefGpuProblem(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dt", C.c_float), ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float),
        ("mu0", C.c_float), ("eps0", C.c_float),
        ("nsources", C.c_int), ("sources", C.POINTER(C.c_int)),
        ("njz", C.c_int), ("jz", C.POINTER(C.c_float)),
        ("media", C.POINTER(C.c_float) * 4), ("rp", C.POINTER(C.c_float) * 6),
    ]


def ref_gpu_available() -> bool:
    """True where the reference kernels were compiled to a cubin (built in a
    container holding the reference sources; the cubin travels with the repo)."""
    return _build.REF_CUBIN.exists()


def _ref_gpu_lib() -> C.CDLL:
    if "ref_gpu" not in _LIBS:
        _build.build_oracle()
        L = C.CDLL(str(_build.REF_GPU_LIB))
        rc = L.ref_gpu_load(str(_build.REF_CUBIN).encode())
        if rc != 0:
            raise RuntimeError(f"ref_gpu_load failed: {rc}")
        _LIBS["ref_gpu"] = L
    return _LIBS["ref_gpu"]


def ref_gpu_run(cfg: OracleCfg, media: Media, nsteps: int, warmup: int = 0, state: State | None = None) -> float:
    """Runs the reference's own CUDA kernels (launch grid, slot rotation and
    step order of fdtd.cu:75-530) for warmup + nsteps steps from zero; fills
    ``state`` (float32) if given and returns the milliseconds of the nsteps
    timed steps.  Step indices must stay below 512 (the reference's dJz)."""
    L = _ref_gpu_lib()
    src, jz = cfg._keep
    keep = [np.ascontiguousarray(a, np.float32) for a in (media.sigma, media.eps_i, media.eps_s, media.tau_d)]
    rps = [np.ascontiguousarray(a, np.float32) for a in media.rp]
    prob = RefGpuProblem(nx=cfg.nx, ny=cfg.ny, nz=cfg.nz, dt=cfg.dt, dx=cfg.dx, dy=cfg.dy, dz=cfg.dz, mu0=cfg.mu0,
                         eps0=cfg.eps0, nsources=cfg.nsources, sources=_ptr(src, C.c_int), njz=len(jz), jz=_ptr(jz))
    for k, a in enumerate(keep):
        prob.media[k] = _ptr(a)
    for k, a in enumerate(rps):
        prob.rp[k] = _ptr(a)
    n = cfg.nx * cfg.ny * cfg.nz
    out = None
    if state is not None:
        assert state.dtype == np.float32
        out = np.empty((21, n), np.float32)
    ms = C.c_float(0.0)
    rc = L.ref_gpu_run(C.byref(prob), warmup, nsteps, None if out is None else _ptr(out), C.byref(ms))
    if rc != 0:
        raise RuntimeError(f"ref_gpu_run failed: {rc}")
    if state is not None:
        for a, src_a in zip(state.arrays(), out):
            a[...] = src_a.reshape(a.shape)
    return float(ms.value)
