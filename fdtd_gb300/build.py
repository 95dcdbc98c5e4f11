"""Build libfdtd_gb300.so (and the drop-in ``fdtd`` executable) in-tree.

Every translation unit is compiled in parallel with nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host code gets
``-ffp-contract=off`` so the set-up arithmetic gives the same bits on x86 and
Arm hosts.  Outputs: ``fdtd_gb300/libfdtd_gb300.so``, ``fdtd_gb300/bin/fdtd``
and ``fdtd_gb300/_build/ptxas.log`` (register and shared-memory report).
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libfdtd_gb300.so"
EXE = PKG / "bin" / "fdtd"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# extra nvcc options, e.g. "-DFDTD_STRIP_STAGES=4" for a build that measures
# another ring depth (a changed value needs a forced rebuild)
EXTRA = os.environ.get("FDTD_NVCC_FLAGS", "").split()

CU_SOURCES = ["compat.cu", "native.cu", "step_fused.cu", "step_strip.cu", "batch_strip.cu", "step_static.cu", "solver.cu", "monitor.cu", "batch.cu", "cuda_util.cu"]
CPP_SOURCES = ["host_io.cpp"]
HEADERS = ["fdtd_internal.h", "device_common.cuh", "native.cuh", "solver_internal.cuh", "tma_util.cuh", "per_device.h", "cell_math.cuh", "strip_unit.cuh"]


def _run(cmd: list[str]) -> str:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    return proc.stdout + proc.stderr


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile what changed; returns the library path."""
    OBJ.mkdir(exist_ok=True)
    (PKG / "bin").mkdir(exist_ok=True)
    common_deps = [CSRC / h for h in HEADERS] + [ROOT / "include" / "fdtd_gb300.h", Path(__file__)]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = OBJ / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + common_deps):
            jobs.append([NVCC, "-c", "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xptxas", "-v",
                         "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{ROOT / 'include'}", *EXTRA,
                         str(CSRC / src), "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = OBJ / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + common_deps):
            jobs.append(["g++", "-c", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                         f"-I{CUDA_HOME / 'include'}", f"-I{ROOT / 'include'}", str(CSRC / src), "-o", str(obj)])
    if jobs:
        with ThreadPoolExecutor(min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
        ptxas = "\n".join(l for l in logs if "ptxas" in l)
        if ptxas:
            (OBJ / "ptxas.log").write_text(ptxas)
        if verbose:
            print("\n".join(logs))
    if force or jobs or _stale(LIB, objs):
        _run([NVCC, "-shared", *ARCH, "-cudart", "shared", "-o", str(LIB), *map(str, objs), "-lpthread"])
    main_src = CSRC / "fdtd_main.cpp"
    if main_src.exists() and (force or _stale(EXE, [main_src, LIB] + common_deps)):
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT / 'include'}", str(main_src), "-o", str(EXE),
              f"-L{PKG}", "-lfdtd_gb300", "-Wl,-rpath,$ORIGIN/..", "-lpthread"])
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
