"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/liboracle_f64.so`` / ``liboracle_f32.so``: the C restatement
  in ``fdtd_oracle.c`` built in FP64 and in the reference's FP32 precision.
* ``oracle/_ref/libref_cpu.so``: the reference's own kernel file compiled as
  C++ for the CPU (``ref/ref_shim_cpu.h`` force-included, ``ref/ref_cpu.cpp``
  loops it over the reference launch grid).
* ``oracle/_ref/libref_host.so``: the reference's host set-up code (params
  parser, source table, voxeliser, snapshot writer) behind C wrappers.
* ``oracle/_ref/ref_kernels.cubin``: the reference's kernel file compiled for
  sm_103a with the reference Makefile's nvcc defaults (device code only, so
  it runs on any host with a GB300).
* ``oracle/_build/libref_gpu.so``: our harness that loads that cubin and
  drives the reference kernels on the GPU (``ref/ref_gpu.cu``); built on every
  host with nvcc, used only where the cubin exists.

The ``_ref`` libraries are built only where the reference sources exist: the
directory ``FDTD_REFERENCE_ROOT`` names, else the build container's mount of
the reference (this recipe is the one file that reads the sources where they
lie).  They compile the reference files in place and write nothing but
``oracle/_ref/``; the GPU machine, which has no reference sources, uses the
files built here.
Both builds use ``-ffp-contract=off`` so x86 and Arm hosts give identical bits.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE_ROOT = Path(os.environ.get("FDTD_REFERENCE_ROOT", "/root/reference"))
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))

ORACLE_LIBS = {"f64": BUILD / "liboracle_f64.so", "f32": BUILD / "liboracle_f32.so"}
REF_CPU_LIB = REF_OUT / "libref_cpu.so"
REF_HOST_LIB = REF_OUT / "libref_host.so"
REF_CUBIN = REF_OUT / "ref_kernels.cubin"
REF_GPU_LIB = BUILD / "libref_gpu.so"


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build_oracle(force: bool = False) -> dict[str, Path]:
    """Compile the C restatement twice (FP64 and FP32)."""
    BUILD.mkdir(exist_ok=True)
    src = HERE / "fdtd_oracle.c"
    jobs = []
    for tag, real in (("f64", "double"), ("f32", "float")):
        out = ORACLE_LIBS[tag]
        if force or _stale(out, [src, Path(__file__)]):
            jobs.append(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
                         "-ffp-contract=off", f"-DORACLE_REAL={real}", str(src), "-o", str(out), "-lm"])
    gpu_src = HERE / "ref" / "ref_gpu.cu"
    nvcc = CUDA_HOME / "bin" / "nvcc"
    if nvcc.exists() and (force or _stale(REF_GPU_LIB, [gpu_src])):
        jobs.append([str(nvcc), "-O2", "-shared", "-Xcompiler", "-fPIC", "-gencode", "arch=compute_103a,code=sm_103a",
                     str(gpu_src), "-o", str(REF_GPU_LIB), f"-L{CUDA_HOME / 'lib64' / 'stubs'}", "-lcuda"])
    with ThreadPoolExecutor(len(jobs) or 1) as ex:
        list(ex.map(_run, jobs))
    return dict(ORACLE_LIBS)


def reference_available() -> bool:
    return (REFERENCE_ROOT / "fdtd_calculations.cu").exists() and (REFERENCE_ROOT / "fdtd.cu").exists()


def build_reference(force: bool = False) -> dict[str, Path] | None:
    """Compile the reference's own sources into oracle/_ref (None if absent)."""
    if not reference_available():
        return None
    REF_OUT.mkdir(exist_ok=True)
    ref = REFERENCE_ROOT
    shim_cpu = HERE / "ref" / "ref_shim_cpu.h"
    shim_host = HERE / "ref" / "ref_shim_host.h"
    deps_cpu = [ref / "fdtd_calculations.cu", ref / "fdtd_calculations.h", shim_cpu, HERE / "ref" / "ref_cpu.cpp"]
    deps_host = [ref / "fdtd.cu", ref / "utils.cu", ref / "fdtd_calculations.cu", shim_host,
                 HERE / "ref" / "ref_host.cu"]

    def cpu() -> None:
        if force or _stale(REF_CPU_LIB, deps_cpu):
            _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-w",
                  "-include", str(shim_cpu), f"-I{ref}", f"-I{CUDA_HOME / 'include'}",
                  str(HERE / "ref" / "ref_cpu.cpp"), "-o", str(REF_CPU_LIB)])

    def host() -> None:
        if not (force or _stale(REF_HOST_LIB, deps_host)):
            return
        nvcc = str(CUDA_HOME / "bin" / "nvcc")
        tmp = REF_OUT / "obj"
        tmp.mkdir(exist_ok=True)
        common = [nvcc, "-c", "-x", "cu", "-O2", "-w", "-Xcompiler", "-fPIC,-ffp-contract=off",
                  "-gencode", "arch=compute_103a,code=sm_103a", f"-I{ref}"]
        objs = []
        units = [(ref / "fdtd.cu", ["-include", str(shim_host), "-Dmain=fdtd_reference_main"]),
                 (ref / "utils.cu", []), (ref / "fdtd_calculations.cu", []),
                 (HERE / "ref" / "ref_host.cu", [])]
        cmds = []
        for src, extra in units:
            obj = tmp / (src.stem + ".o")
            objs.append(obj)
            cmds.append(common + extra + [str(src), "-o", str(obj)])
        with ThreadPoolExecutor(len(cmds)) as ex:
            list(ex.map(_run, cmds))
        _run([nvcc, "-shared", "-o", str(REF_HOST_LIB)] + [str(o) for o in objs])
        shutil.rmtree(tmp, ignore_errors=True)

    def cubin() -> None:
        # the reference Makefile's nvcc invocation (no optimisation or
        # fast-math options) with the GB300 target; device code only
        if force or _stale(REF_CUBIN, [ref / "fdtd_calculations.cu", ref / "fdtd_calculations.h"]):
            _run([str(CUDA_HOME / "bin" / "nvcc"), "-cubin", "-w", "-gencode", "arch=compute_103a,code=sm_103a",
                  f"-I{ref}", str(ref / "fdtd_calculations.cu"), "-o", str(REF_CUBIN)])

    with ThreadPoolExecutor(3) as ex:
        for f in [ex.submit(cpu), ex.submit(host), ex.submit(cubin)]:
            f.result()
    return {"cpu": REF_CPU_LIB, "host": REF_HOST_LIB, "cubin": REF_CUBIN}


def build(force: bool = False) -> None:
    build_oracle(force)
    build_reference(force)


if __name__ == "__main__":
    build(force=True)
    print("oracle:", ORACLE_LIBS, "reference:", REF_CPU_LIB if reference_available() else "absent")
