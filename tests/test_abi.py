"""The C-ABI library loads and exports every entry point its header declares."""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

import numpy as np

import fdtd_gb300 as fg

HEADER_DIR = Path(__file__).resolve().parent.parent / "include"


def declared_functions() -> set[str]:
    names = set()
    for h in HEADER_DIR.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"typedef[^;]*;", "", text)
        names |= set(re.findall(r"\b(fdtd_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_function():
    names = declared_functions()
    assert len(names) >= 30
    L = fg.lib()
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(fg.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (fdtd_[a-z0-9_]+)\b", out))
    assert names <= exported, sorted(names - exported)


def test_status_strings():
    L = fg.lib()
    assert L.fdtd_status_string(0) == b"success"
    assert b"format" in L.fdtd_status_string(fg.FDTD_ERR_FORMAT)
    assert L.fdtd_status_string(2)  # a CUDA error code


def test_invalid_arguments_return_status_without_a_gpu():
    L = fg.lib()
    assert L.fdtd_params_read(None, None) == fg.FDTD_ERR_INVALID
    assert L.fdtd_setup_sources(None) == fg.FDTD_ERR_INVALID
    assert L.fdtd_plan_create(None, None, 0, 0, None, None) == fg.FDTD_ERR_INVALID
    assert L.fdtd_solver_create(None, None) == fg.FDTD_ERR_INVALID
    assert L.fdtd_step(None, None, 0, None) == fg.FDTD_ERR_INVALID


def test_plan_parameters_checked_before_any_device_call():
    """fdtd_plan_create refuses a bad grid, source, scheme or class count
    with FDTD_ERR_INVALID before it touches the device (so without a GPU)."""
    import ctypes as C

    L = fg.lib()
    specs = np.zeros((2, 4), np.float32)
    specs[:, 1:3] = 1.0
    src = (C.c_int * 3)(5, 5, 5)

    def params(nx=16, ny=16, nz=16, sources=(5, 5, 5)):
        raw = fg.FdtdParams()
        raw.nx, raw.ny, raw.nz = nx, ny, nz
        src[:] = sources
        raw.sourcesCount, raw.sources = 1, C.cast(src, C.POINTER(C.c_int))
        raw.dt, raw.dx, raw.dy, raw.dz, raw.mu0, raw.eps0 = 1.9e-12, 1e-3, 1e-3, 1e-3, 1.2566371e-06, 8.85e-12
        return raw

    h = C.c_void_p()
    sp = specs.ctypes.data_as(C.POINTER(C.c_float))
    for raw, ncls, scheme in [(params(nx=2), 2, 0), (params(nz=70000), 2, 0), (params(sources=(0, 5, 5)), 2, 0),
                              (params(sources=(5, 16, 5)), 2, 0), (params(sources=(5, 5, 16)), 2, 0),
                              (params(), 2, 7), (params(), 0, 0), (params(), fg.MAX_CLASSES + 1, 0)]:
        assert L.fdtd_plan_create(C.byref(raw), sp, ncls, scheme, None, C.byref(h)) == fg.FDTD_ERR_INVALID
        assert not h.value


def test_drop_in_executable_built_and_reports_usage():
    import subprocess

    assert fg.EXE_PATH.exists()
    r = subprocess.run([str(fg.EXE_PATH), "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([str(fg.EXE_PATH), "--params", "/nonexistent/input_params"], capture_output=True, text=True)
    assert r.returncode == 1 and "failed" in r.stderr


def test_kernel_form_ids_match_the_header():
    """The Python mirror's form ids are the header's enum values."""
    text = (HEADER_DIR / "fdtd_gb300.h").read_text()
    ids = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(FDTD_KERNEL_[A-Z0-9_]+)\s*=\s*(\d+)", text)}
    assert ids == {"FDTD_KERNEL_SINGLE_PASS": fg.KERNEL_SINGLE_PASS, "FDTD_KERNEL_TWO_PASS": fg.KERNEL_TWO_PASS,
                   "FDTD_KERNEL_COMPACT": fg.KERNEL_COMPACT, "FDTD_KERNEL_COMPACT_R16": fg.KERNEL_COMPACT_R16}
    assert set(fg.COMPACT_KERNELS) == {fg.KERNEL_COMPACT, fg.KERNEL_COMPACT_R16}


def test_field_output_buffer_checked_before_the_library_call():
    """Solver.field(name, out=...) refuses a buffer of the wrong shape, type or
    layout before it calls the library (host logic; no solver is created)."""
    s = fg.Solver.__new__(fg.Solver)  # only the attributes field() reads first
    s.params = type("P", (), {"shape": (4, 5, 6)})()
    s.handle = None
    for bad in (np.empty((4, 5, 7), np.float32), np.empty((4, 5, 6), np.float64),
                np.empty((6, 5, 4), np.float32).transpose(2, 1, 0)):
        with np.testing.assert_raises(ValueError):
            s.field("ez", out=bad)
