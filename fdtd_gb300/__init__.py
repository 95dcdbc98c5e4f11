"""fdtd_gb300 -- GB300-native 3-D Yee FDTD (Debye media, Mur boundaries).

Python mirror of the C ABI in ``include/fdtd_gb300.h`` (libfdtd_gb300.so).
The compute path is the CUDA library; this module only binds it.  Loading
fails loudly when the library has not been built (``fdtd_gb300.build``):
there is no CPU fallback.

Reference correspondence (rafalgrodzinski/fdtd):
  params_read          initParamsWithPath   fdtd.cu:547-637
  Params.setup_sources setupSources         fdtd.cu:1027-1082
  setup_mur            setupMurBoundary     fdtd.cu:942-1024
  load_materials       loadMaterials        fdtd.cu:875-939
  write_results3d      writeResults3d       fdtd.cu:1288-1494
  copy_symbols, update_h/d/e/sources/mur    fdtd_calculations.h:18-42
  Solver               the time loop        fdtd.cu:115-530
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libfdtd_gb300.so"
EXE_PATH = _PKG / "bin" / "fdtd"

FDTD_OK = 0
FDTD_ERR_INVALID = 10001
FDTD_ERR_IO = 10002
FDTD_ERR_FORMAT = 10003
FDTD_ERR_NO_SYMBOLS = 10004
FDTD_ERR_NOMEM = 10005
FDTD_ERR_STATE = 10006
FDTD_ERR_DEVICE_TIMEOUT = 10007
FDTD_ERR_BUSY = 10008
MAX_SOURCES = 16
JZ_LEN = 65536
MAX_CLASSES = 256
STATIC_MAX_CLASSES = 64
SCHEME_REFERENCE = 0
SCHEME_CORRECTED = 1
KERNEL_SINGLE_PASS = 0
KERNEL_TWO_PASS = 1
KERNEL_COMPACT = 2      # nine stored fields (H, E, R); D is not readable
KERNEL_COMPACT_R16 = 3  # the same with R in 16 bits (FP16 residual + one scale per 32-cell row segment)
COMPACT_KERNELS = (KERNEL_COMPACT, KERNEL_COMPACT_R16)
FIELDS = ("hx", "hy", "hz", "dx", "dy", "dz", "ex", "ey", "ez")
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}


class FdtdError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        text = lib().fdtd_status_string(status).decode() if _LIB is not None else str(status)
        super().__init__(f"{what}: status {status} ({text})" if what else f"status {status} ({text})")


class FdtdParams(C.Structure):
    """Same members, types and order as the reference's FdtdParams (fdtd.h:7-34)."""

    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("iterationsCount", C.c_int),
        ("inputPath", C.c_char_p), ("outputPath", C.c_char_p), ("elementsPerWave", C.c_int),
        ("waveFrequency", C.c_float), ("pulseWidth", C.c_float), ("pulseModulationFrequency", C.c_float),
        ("sourcesCount", C.c_int), ("sources", C.POINTER(C.c_int)),
        ("defaultSigma", C.c_float), ("defaultEpsS", C.c_float), ("defaultEpsI", C.c_float),
        ("defaultTauD", C.c_float), ("jzCount", C.c_int), ("jz", C.POINTER(C.c_float)),
        ("pi", C.c_float), ("c", C.c_float), ("timeskip", C.c_float), ("lambda_", C.c_float),
        ("dt", C.c_float), ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float),
        ("mu0", C.c_float), ("eps0", C.c_float),
    ]


class NativeFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "hx", "hy", "hz", "hx_out", "hy_out", "hz_out", "ex", "ey", "ez", "ex_prev", "ey_prev", "ez_prev",
        "dx", "dy", "dz", "dx_prev", "dy_prev", "dz_prev", "material")]


class SolverConfig(C.Structure):
    _fields_ = [("params", C.POINTER(FdtdParams)), ("material", C.POINTER(C.c_uint8)),
                ("specs", C.POINTER(C.c_float)), ("nclasses", C.c_int), ("scheme", C.c_int),
                ("kernel", C.c_int), ("device", C.c_int)]


SNAPSHOT_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_int, C.c_int)


class SnapshotSpec(C.Structure):
    _fields_ = [("every", C.c_int), ("field_mask", C.c_uint32), ("z0", C.c_int), ("nplanes", C.c_int),
                ("callback", SNAPSHOT_FN), ("user", C.c_void_p), ("output_dir", C.c_char_p),
                ("writer_threads", C.c_int), ("format", C.c_int)]

SNAPSHOT_TEXT, SNAPSHOT_BINARY, SNAPSHOT_TEXT_AND_BINARY = 0, 1, 2


_LIB: C.CDLL | None = None

_P = C.POINTER(C.c_float)
_V = C.c_void_p
_I = C.c_int


def _sig(L, name, restype, *argtypes):
    f = getattr(L, name)
    f.restype = restype
    f.argtypes = list(argtypes)


def lib() -> C.CDLL:
    """The loaded library; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        path = Path(os.environ.get("FDTD_GB300_LIB", LIB_PATH))
        if not path.exists():
            raise FileNotFoundError(f"{path} is missing: build it with `python -m fdtd_gb300.build`")
        L = C.CDLL(str(path))
        PP = C.POINTER(FdtdParams)
        _sig(L, "fdtd_status_string", C.c_char_p, _I)
        _sig(L, "fdtd_params_read", _I, C.c_char_p, PP)
        _sig(L, "fdtd_params_set_timeskip", _I, PP, C.c_float)
        _sig(L, "fdtd_params_free", None, PP)
        _sig(L, "fdtd_setup_sources", _I, PP)
        _sig(L, "fdtd_setup_mur", _I, PP, *([_P] * 10))
        _sig(L, "fdtd_setup_mur_uniform", _I, PP, C.c_float, C.c_float, C.c_float, C.c_float, *([_P] * 6))
        _sig(L, "fdtd_read_specs", _I, C.c_char_p, _P)
        _sig(L, "fdtd_load_material_codes", _I, PP, C.c_char_p, C.POINTER(C.c_uint8), _I)
        _sig(L, "fdtd_load_material_codes_cached", _I, PP, C.c_char_p, C.c_char_p, C.POINTER(C.c_uint8), _I,
             C.POINTER(_I))
        _sig(L, "fdtd_load_materials", _I, PP, C.c_char_p, C.c_char_p, *([_P] * 4))
        _sig(L, "fdtd_write_results3d", _I, PP, *([_P] * 9), _I, _I)
        _sig(L, "fdtd_copy_symbols", _I, PP)
        _sig(L, "fdtd_update_h", _I, *([_V] * 6), _V)
        _sig(L, "fdtd_update_d", _I, *([_V] * 9), _V)
        _sig(L, "fdtd_update_e", _I, *([_V] * 22), _V)
        _sig(L, "fdtd_update_sources", _I, _V, _V, _V, _V, _I, _V)
        _sig(L, "fdtd_update_mur", _I, *([_V] * 12), _V)
        _sig(L, "fdtd_plan_create", _I, PP, _P, _I, _I, C.POINTER(_P), C.POINTER(_V))
        _sig(L, "fdtd_plan_destroy", _I, _V)
        _sig(L, "fdtd_plan_status", _I, _V)
        _sig(L, "fdtd_step_h", _I, _V, C.POINTER(NativeFields), _V)
        _sig(L, "fdtd_step_de", _I, _V, C.POINTER(NativeFields), _I, _V)
        _sig(L, "fdtd_step", _I, _V, C.POINTER(NativeFields), _I, _V)
        _sig(L, "fdtd_step_static", _I, PP, _P, _I, _I, C.POINTER(NativeFields), C.POINTER(_V), _I, _V)
        _sig(L, "fdtd_solver_create", _I, C.POINTER(SolverConfig), C.POINTER(_V))
        _sig(L, "fdtd_solver_destroy", _I, _V)
        _sig(L, "fdtd_solver_run", _I, _V, _I)
        _sig(L, "fdtd_solver_synchronize", _I, _V)
        _sig(L, "fdtd_solver_test_stall", _I, _V)
        _sig(L, "fdtd_solver_steps", _I, _V)
        _sig(L, "fdtd_solver_get_field", _I, _V, _I, _P)
        _sig(L, "fdtd_solver_stream", _V, _V)
        _sig(L, "fdtd_solver_set_snapshots", _I, _V, C.POINTER(SnapshotSpec))
        _sig(L, "fdtd_solver_flush_snapshots", _I, _V)
        _sig(L, "fdtd_solver_profile", _I, _V, _I, _P, _I, C.POINTER(_I))
        _sig(L, "fdtd_solver_checkpoint", _I, _V, C.c_char_p)
        _sig(L, "fdtd_solver_restore", _I, _V, C.c_char_p)
        _sig(L, "fdtd_solver_set_probes", _I, _V, _I, C.POINTER(_I), _I)
        _sig(L, "fdtd_solver_get_probes", _I, _V, _P, C.POINTER(_I))
        _sig(L, "fdtd_solver_set_dft", _I, _V, C.c_double, _I, _I, _I)
        _sig(L, "fdtd_solver_get_dft", _I, _V, _I, C.POINTER(C.c_double), C.POINTER(C.c_double))
        _sig(L, "fdtd_solver_peak_sar", _I, _V, _P, C.POINTER(C.c_double), C.POINTER(C.c_longlong))
        _sig(L, "fdtd_solver_kernel_name", C.c_char_p, _V, _I)
        _sig(L, "fdtd_solver_memless_fraction", C.c_double, _V)
        _sig(L, "fdtd_batch_create", _I, _I, C.POINTER(_V))
        _sig(L, "fdtd_batch_create_form", _I, _I, _I, C.POINTER(_V))
        _sig(L, "fdtd_batch_need_bytes", C.c_size_t, _V, _I, _I, _I)
        _sig(L, "fdtd_batch_destroy", _I, _V)
        _sig(L, "fdtd_batch_solve_bytes", C.c_size_t, _I, _I, _I)
        _sig(L, "fdtd_batch_add", _I, _V, C.POINTER(SolverConfig), _I, C.POINTER(_I))
        _sig(L, "fdtd_batch_remove", _I, _V, _I)
        _sig(L, "fdtd_batch_run", _I, _V, _I)
        _sig(L, "fdtd_batch_synchronize", _I, _V)
        _sig(L, "fdtd_batch_autotune", _I, _V, _I, C.POINTER(_I))
        _sig(L, "fdtd_batch_tuning", _I, _V, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I))
        _sig(L, "fdtd_batch_steps", _I, _V, _I)
        _sig(L, "fdtd_batch_get_field", _I, _V, _I, _I, _I, _I, _P)
        _sig(L, "fdtd_batch_bytes", C.c_size_t, _V)
        _sig(L, "fdtd_batch_size", _I, _V)
        _sig(L, "fdtd_batch_stream", _V, _V)
        _sig(L, "fdtd_batch_read_async", _I, _V, _I, _I, _I, _I, _V, C.POINTER(C.c_longlong))
        _sig(L, "fdtd_batch_mark", _I, _V, C.POINTER(C.c_longlong))
        _sig(L, "fdtd_batch_ticket", _I, _V, C.c_longlong, _I)
        _sig(L, "fdtd_batch_set_timing", _I, _V, _I)
        _sig(L, "fdtd_batch_busy", _I, _V, C.POINTER(C.c_double), C.POINTER(C.c_double))
        _sig(L, "fdtd_host_alloc", _I, C.c_size_t, C.POINTER(_V))
        _sig(L, "fdtd_host_free", _I, _V)
        _LIB = L
    return _LIB


def check(status: int, what: str = "") -> None:
    if status != FDTD_OK:
        raise FdtdError(status, what)


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


# ----------------------------------------------------------------- params

class Params:
    """Owns a FdtdParams filled by the library (freed on close)."""

    def __init__(self, raw: FdtdParams):
        self.raw = raw

    @classmethod
    def read(cls, path: str | os.PathLike) -> "Params":
        raw = FdtdParams()
        check(lib().fdtd_params_read(str(path).encode(), C.byref(raw)), f"fdtd_params_read({path})")
        return cls(raw)

    def set_timeskip(self, timeskip: float) -> None:
        check(lib().fdtd_params_set_timeskip(C.byref(self.raw), timeskip), "fdtd_params_set_timeskip")

    def setup_sources(self) -> np.ndarray:
        check(lib().fdtd_setup_sources(C.byref(self.raw)), "fdtd_setup_sources")
        return self.jz

    @property
    def jz(self) -> np.ndarray | None:
        if not self.raw.jz:
            return None
        return np.ctypeslib.as_array(self.raw.jz, shape=(self.raw.jzCount,)).copy()

    @property
    def sources(self) -> list[tuple[int, int, int]]:
        r = self.raw
        return [(r.sources[3 * k], r.sources[3 * k + 1], r.sources[3 * k + 2]) for k in range(r.sourcesCount)]

    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.raw.nz, self.raw.ny, self.raw.nx)

    def __getattr__(self, name):
        return getattr(self.raw, name)

    def close(self) -> None:
        if self.raw is not None:
            lib().fdtd_params_free(C.byref(self.raw))
            self.raw = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def params_read(path) -> Params:
    return Params.read(path)


def rp_shapes(nx: int, ny: int, nz: int) -> list[tuple[int, int, int]]:
    """Mur slab shapes (C order): rpx0, rpy0, rpz0, rpxEnd, rpyEnd, rpzEnd."""
    return [(nz, ny, 2), (nz, 2, nx), (2, ny, nx)] * 2


def setup_mur(p: Params, sigma, eps_s, eps_i, tau) -> list[np.ndarray]:
    rp = [np.zeros(s, np.float32) for s in rp_shapes(p.nx, p.ny, p.nz)]
    check(lib().fdtd_setup_mur(C.byref(p.raw), fptr(sigma), fptr(eps_s), fptr(eps_i), fptr(tau),
                               *[fptr(r) for r in rp]), "fdtd_setup_mur")
    return rp


def setup_mur_uniform(p: Params, sigma: float, eps_s: float, eps_i: float, tau: float) -> list[np.ndarray]:
    rp = [np.zeros(s, np.float32) for s in rp_shapes(p.nx, p.ny, p.nz)]
    check(lib().fdtd_setup_mur_uniform(C.byref(p.raw), sigma, eps_s, eps_i, tau, *[fptr(r) for r in rp]),
          "fdtd_setup_mur_uniform")
    return rp


def read_specs(path) -> np.ndarray:
    specs = np.zeros((MAX_CLASSES, 4), np.float32)
    check(lib().fdtd_read_specs(str(path).encode(), fptr(specs)), f"fdtd_read_specs({path})")
    return specs


def load_material_codes(p: Params, pgm_dir, nthreads: int = 0, cache=None) -> np.ndarray:
    """uint8 class volume from the PGM slices; with `cache` (a file path),
    through the binary cache (see load_material_codes_cached)."""
    if cache is not None:
        return load_material_codes_cached(p, pgm_dir, cache, nthreads)[0]
    codes = np.zeros(p.shape, np.uint8)
    check(lib().fdtd_load_material_codes(C.byref(p.raw), str(pgm_dir).encode(),
                                         codes.ctypes.data_as(C.POINTER(C.c_uint8)), nthreads),
          "fdtd_load_material_codes")
    return codes


def load_material_codes_cached(p: Params, pgm_dir, cache, nthreads: int = 0) -> tuple[np.ndarray, bool]:
    """(class volume, whether it came from the cache file)."""
    codes = np.zeros(p.shape, np.uint8)
    hit = C.c_int(0)
    check(lib().fdtd_load_material_codes_cached(C.byref(p.raw), str(pgm_dir).encode(), str(cache).encode(),
                                                codes.ctypes.data_as(C.POINTER(C.c_uint8)), nthreads,
                                                C.byref(hit)), "fdtd_load_material_codes_cached")
    return codes, bool(hit.value)


def load_materials(p: Params, specs_path, pgm_dir) -> tuple[np.ndarray, ...]:
    """(sigma, eps_s, eps_i, tau) per cell, as loadMaterials fills them."""
    arrs = [np.zeros(p.shape, np.float32) for _ in range(4)]
    check(lib().fdtd_load_materials(C.byref(p.raw), str(specs_path).encode(), str(pgm_dir).encode(),
                                    *[fptr(a) for a in arrs]), "fdtd_load_materials")
    return tuple(arrs)


def write_results3d(p: Params, fields: dict, iteration: int, nthreads: int = 0) -> None:
    arrs = []
    for n in FIELDS:
        a = fields.get(n)
        arrs.append(None if a is None else np.ascontiguousarray(a, np.float32))
    ptrs = [fptr(a) if a is not None else None for a in arrs]
    check(lib().fdtd_write_results3d(C.byref(p.raw), *ptrs, iteration, nthreads), "fdtd_write_results3d")


# ---------------------------------------------------------------- solver

class Solver:
    """One resident solve on one GPU (fdtd_solver_*)."""

    def __init__(self, p: Params, material: np.ndarray, specs: np.ndarray, scheme: int = SCHEME_REFERENCE,
                 kernel: int = KERNEL_SINGLE_PASS, device: int = 0, nclasses: int | None = None):
        self.params = p
        self.material = np.ascontiguousarray(material, np.uint8)
        specs = np.ascontiguousarray(specs, np.float32).reshape(-1, 4)
        if nclasses is None:
            # every row given; the library keeps those up to the largest class present
            nclasses = min(len(specs), MAX_CLASSES)
        self.specs = np.ascontiguousarray(specs[:nclasses])
        cfg = SolverConfig(params=C.pointer(p.raw), material=self.material.ctypes.data_as(C.POINTER(C.c_uint8)),
                           specs=fptr(self.specs), nclasses=nclasses, scheme=scheme, kernel=kernel, device=device)
        h = C.c_void_p()
        check(lib().fdtd_solver_create(C.byref(cfg), C.byref(h)), "fdtd_solver_create")
        self.handle = h
        self.kernel = kernel
        self._cb = None
        self._spec = None

    def run(self, nsteps: int) -> None:
        check(lib().fdtd_solver_run(self.handle, nsteps), "fdtd_solver_run")

    def synchronize(self) -> None:
        check(lib().fdtd_solver_synchronize(self.handle), "fdtd_solver_synchronize")

    def test_stall(self) -> None:
        """Failure-path test hook: the next single-pass step's first CTA lets one
        bounded wait run out; synchronize() then raises FDTD_ERR_DEVICE_TIMEOUT."""
        check(lib().fdtd_solver_test_stall(self.handle), "fdtd_solver_test_stall")

    @property
    def steps(self) -> int:
        return lib().fdtd_solver_steps(self.handle)

    @property
    def stream(self) -> int:
        return lib().fdtd_solver_stream(self.handle) or 0

    def field(self, name: str, out: np.ndarray | None = None) -> np.ndarray:
        """One field volume (nz, ny, nx) float32; into `out` when given (a
        reused buffer skips the first-touch cost of fresh host pages)."""
        if out is None:
            out = np.empty(self.params.shape, np.float32)
        elif out.shape != self.params.shape or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous float32 array of shape {self.params.shape}")
        check(lib().fdtd_solver_get_field(self.handle, FIELD_ID[name], fptr(out)), "fdtd_solver_get_field")
        return out

    def fields(self) -> dict[str, np.ndarray]:
        """Every stored field (the compact form stores no D)."""
        names = [n for n in FIELDS if not (self.kernel in COMPACT_KERNELS and n.startswith("d"))]
        return {n: self.field(n) for n in names}

    def set_snapshots(self, every: int, fields=("ex", "ey", "ez"), z0: int = 0, nplanes: int = 0,
                      callback=None, output_dir: str | None = None, writer_threads: int = 0,
                      format: int = SNAPSHOT_TEXT) -> None:
        """Snapshots every `every` steps to `callback(step, name, planes)`, or to
        files under output_dir: the reference text layout (SNAPSHOT_TEXT), raw
        float32 files (SNAPSHOT_BINARY) or both."""
        mask = 0
        for n in fields:
            mask |= 1 << FIELD_ID[n]
        cb = SNAPSHOT_FN() if callback is None else SNAPSHOT_FN(
            lambda user, step, field, data, z0_, np_: callback(
                step, FIELDS[field], np.ctypeslib.as_array(data, shape=(np_, self.params.ny, self.params.nx)).copy()))
        spec = SnapshotSpec(every=every, field_mask=mask, z0=z0, nplanes=nplanes, callback=cb, user=None,
                            output_dir=None if output_dir is None else str(output_dir).encode(),
                            writer_threads=writer_threads, format=format)
        check(lib().fdtd_solver_set_snapshots(self.handle, C.byref(spec)), "fdtd_solver_set_snapshots")
        self._cb, self._spec = cb, spec

    def profile(self, nsteps: int) -> dict[str, float]:
        """Average milliseconds per launch of each kernel of a step."""
        ms = (C.c_float * 8)()
        nk = C.c_int()
        check(lib().fdtd_solver_profile(self.handle, nsteps, ms, 8, C.byref(nk)), "fdtd_solver_profile")
        return {lib().fdtd_solver_kernel_name(self.handle, k).decode(): float(ms[k]) for k in range(nk.value)}

    @property
    def memless_fraction(self) -> float:
        """Compact forms: share of the cell-updates on tile-planes without Debye
        memory, whose R the step kernel skips."""
        return lib().fdtd_solver_memless_fraction(self.handle)

    def checkpoint(self, path) -> None:
        check(lib().fdtd_solver_checkpoint(self.handle, str(path).encode()), "fdtd_solver_checkpoint")

    def restore(self, path) -> None:
        check(lib().fdtd_solver_restore(self.handle, str(path).encode()), "fdtd_solver_restore")

    def set_probes(self, cells, capacity: int) -> None:
        xyz = np.ascontiguousarray(np.array(cells, np.int32).reshape(-1))
        check(lib().fdtd_solver_set_probes(self.handle, xyz.size // 3, xyz.ctypes.data_as(C.POINTER(C.c_int)),
                                           capacity), "fdtd_solver_set_probes")
        self._nprobes, self._probe_cap = xyz.size // 3, capacity

    def probes(self) -> np.ndarray:
        """(steps, nprobes, 3) E series since the probes were installed."""
        out = np.zeros((self._probe_cap, self._nprobes, 3), np.float32)
        n = C.c_int()
        check(lib().fdtd_solver_get_probes(self.handle, fptr(out), C.byref(n)), "fdtd_solver_get_probes")
        return out[: n.value]

    def set_dft(self, frequency: float, stride: int = 1, z0: int = 0, nplanes: int = 0) -> None:
        check(lib().fdtd_solver_set_dft(self.handle, frequency, stride, z0, nplanes), "fdtd_solver_set_dft")
        self._dft_np = nplanes or self.params.nz

    def dft(self, comp: int) -> np.ndarray:
        """Complex (nplanes, ny, nx) accumulator of E component comp."""
        shape = (self._dft_np, self.params.ny, self.params.nx)
        re = np.zeros(shape, np.float64)
        im = np.zeros(shape, np.float64)
        P = C.POINTER(C.c_double)
        check(lib().fdtd_solver_get_dft(self.handle, comp, re.ctypes.data_as(P), im.ctypes.data_as(P)),
              "fdtd_solver_get_dft")
        return re + 1j * im

    def peak_sar(self, rho=None) -> tuple[float, int]:
        peak = C.c_double()
        cell = C.c_longlong()
        r = None if rho is None else fptr(np.ascontiguousarray(rho, np.float32))
        check(lib().fdtd_solver_peak_sar(self.handle, r, C.byref(peak), C.byref(cell)), "fdtd_solver_peak_sar")
        return peak.value, cell.value

    def flush_snapshots(self) -> None:
        check(lib().fdtd_solver_flush_snapshots(self.handle), "fdtd_solver_flush_snapshots")

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().fdtd_solver_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------- batch

class Batch:
    """Many independent solves advanced together (fdtd_batch_*)."""

    def __init__(self, device: int = 0, kernel: int = KERNEL_SINGLE_PASS):
        """kernel: KERNEL_SINGLE_PASS (D form), KERNEL_COMPACT or KERNEL_COMPACT_R16 for
        every solve."""
        h = C.c_void_p()
        check(lib().fdtd_batch_create_form(device, kernel, C.byref(h)), "fdtd_batch_create_form")
        self.handle = h
        self.kernel = kernel
        self._keep = {}

    @staticmethod
    def solve_bytes(nx: int, ny: int, nz: int) -> int:
        """Device bytes of one D-form solve."""
        return lib().fdtd_batch_solve_bytes(nx, ny, nz)

    def need_bytes(self, nx: int, ny: int, nz: int) -> int:
        """Device bytes of one solve of this batch's form."""
        return lib().fdtd_batch_need_bytes(self.handle, nx, ny, nz)

    def add(self, p: Params, material: np.ndarray, specs: np.ndarray, steps: int,
            scheme: int = SCHEME_REFERENCE, nclasses: int | None = None) -> int:
        material = np.ascontiguousarray(material, np.uint8)
        specs = np.ascontiguousarray(specs, np.float32).reshape(-1, 4)
        if nclasses is None:
            nclasses = min(len(specs), MAX_CLASSES)
        specs = np.ascontiguousarray(specs[:nclasses])
        cfg = SolverConfig(params=C.pointer(p.raw), material=material.ctypes.data_as(C.POINTER(C.c_uint8)),
                           specs=fptr(specs), nclasses=nclasses, scheme=scheme, kernel=0, device=0)
        sid = C.c_int()
        check(lib().fdtd_batch_add(self.handle, C.byref(cfg), steps, C.byref(sid)), "fdtd_batch_add")
        self._keep[sid.value] = (p, (p.raw.nz, p.raw.ny, p.raw.nx))
        return sid.value

    def remove(self, sid: int) -> None:
        check(lib().fdtd_batch_remove(self.handle, sid), "fdtd_batch_remove")
        self._keep.pop(sid, None)

    def run(self, nsteps: int) -> None:
        check(lib().fdtd_batch_run(self.handle, nsteps), "fdtd_batch_run")

    def synchronize(self) -> None:
        check(lib().fdtd_batch_synchronize(self.handle), "fdtd_batch_synchronize")

    def autotune(self, steps_per_trial: int = 16) -> int:
        """Times each candidate z-chunk limit on the current solves (the trial
        steps are real steps) and keeps the fastest; returns it (0: default)."""
        chosen = C.c_int(0)
        check(lib().fdtd_batch_autotune(self.handle, steps_per_trial, C.byref(chosen)), "fdtd_batch_autotune")
        return chosen.value

    def tuning(self) -> dict:
        """The launch shape in use: z-chunk limit (0: default), tile rows and
        the strip kernel's shape (-1: D form)."""
        z, r, sh = C.c_int(), C.c_int(), C.c_int()
        check(lib().fdtd_batch_tuning(self.handle, C.byref(z), C.byref(r), C.byref(sh)), "fdtd_batch_tuning")
        return {"z_chunk_limit": z.value, "tile_rows": r.value, "strip_shape": sh.value}

    def steps(self, sid: int) -> int:
        return lib().fdtd_batch_steps(self.handle, sid)

    def field(self, sid: int, name: str, z0: int = 0, nplanes: int = 0) -> np.ndarray:
        nz, ny, nx = self._keep[sid][1]
        out = np.empty((nplanes or nz, ny, nx), np.float32)
        check(lib().fdtd_batch_get_field(self.handle, sid, FIELD_ID[name], z0, nplanes, fptr(out)),
              "fdtd_batch_get_field")
        return out

    def fields(self, sid: int) -> dict[str, np.ndarray]:
        names = [n for n in FIELDS if not (self.kernel in COMPACT_KERNELS and n.startswith("d"))]
        return {n: self.field(sid, n) for n in names}

    def read_async(self, sid: int, name: str, out: np.ndarray, z0: int = 0, nplanes: int = 0) -> int:
        """Queues a copy of planes [z0, z0 + nplanes) of a field, as it will be
        after the steps queued so far, into out (float32, (nplanes, ny, nx);
        page-locked for an asynchronous copy, e.g. PinnedBuffer); returns a
        ticket for done().  out must stay alive until then."""
        nz, ny, nx = self._keep[sid][1]
        n = nplanes or nz
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size >= n * ny * nx
        t = C.c_longlong()
        check(lib().fdtd_batch_read_async(self.handle, sid, FIELD_ID[name], z0, nplanes,
                                          out.ctypes.data_as(C.c_void_p), C.byref(t)), "fdtd_batch_read_async")
        return t.value

    def mark(self) -> int:
        """A ticket for the point after everything queued so far."""
        t = C.c_longlong()
        check(lib().fdtd_batch_mark(self.handle, C.byref(t)), "fdtd_batch_mark")
        return t.value

    def done(self, ticket: int, wait: bool = False) -> bool:
        """Whether the ticket's work has finished (the ticket is then spent)."""
        st = lib().fdtd_batch_ticket(self.handle, ticket, 1 if wait else 0)
        if st == FDTD_ERR_BUSY:
            return False
        check(st, "fdtd_batch_ticket")
        return True

    def set_timing(self, on: bool = True) -> None:
        check(lib().fdtd_batch_set_timing(self.handle, 1 if on else 0), "fdtd_batch_set_timing")

    def busy(self) -> tuple[float, float]:
        """(GPU ms of the finished timed runs, ms from the first run's start to
        the last finished run's end)."""
        b, s = C.c_double(), C.c_double()
        check(lib().fdtd_batch_busy(self.handle, C.byref(b), C.byref(s)), "fdtd_batch_busy")
        return b.value, s.value

    @property
    def bytes(self) -> int:
        return lib().fdtd_batch_bytes(self.handle)

    @property
    def stream(self) -> int:
        return lib().fdtd_batch_stream(self.handle) or 0

    def __len__(self) -> int:
        return lib().fdtd_batch_size(self.handle)

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().fdtd_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedBuffer:
    """Page-locked host memory (fdtd_host_alloc) viewed as a float32 array,
    for asynchronous device-to-host copies."""

    def __init__(self, nfloats: int):
        p = C.c_void_p()
        check(lib().fdtd_host_alloc(4 * nfloats, C.byref(p)), "fdtd_host_alloc")
        self._ptr = p
        self.array = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_float)), shape=(nfloats,))

    def view(self, shape) -> np.ndarray:
        n = int(np.prod(shape))
        return self.array[:n].reshape(shape)

    def close(self) -> None:
        if getattr(self, "_ptr", None):
            self.array = None
            lib().fdtd_host_free(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------- native plan API

class Plan:
    """fdtd_plan: device-resident constants of the native kernels."""

    def __init__(self, p: Params, specs: np.ndarray, scheme: int = SCHEME_REFERENCE, rp=None):
        specs = np.ascontiguousarray(specs, np.float32).reshape(-1, 4)
        self._specs = specs
        rp_arr = None
        if rp is not None:
            self._rp = [np.ascontiguousarray(r, np.float32) for r in rp]
            rp_arr = (_P * 6)(*[fptr(r) for r in self._rp])
        h = C.c_void_p()
        check(lib().fdtd_plan_create(C.byref(p.raw), fptr(specs), len(specs), scheme, rp_arr, C.byref(h)),
              "fdtd_plan_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            lib().fdtd_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
