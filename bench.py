#!/usr/bin/env python3
"""Benchmark: Yee cell-updates per second on the 512 x 512 x 400 phantom.

Workload: 8 nested, seeded ellipsoids of Debye tissue in vacuum (uint8 class
volume), a 900 MHz three-cell Ez dipole 20 cells outside the outer shell,
Mur faces, dx = 1 mm, dt = 0.99 of the Courant limit, corrected scheme (the
reference scheme doubles |E| every step in vacuum; both schemes run the same
kernels at the same speed), FP32 fields.  One step is one full Yee step (H,
D + sources, Debye E, Mur) over all 104,857,600 cells.  The state (7.6 GB)
is far larger than L2, so no flush is needed between steps.

Default arm (``--impl gb300``): the library's solver, steps replayed as CUDA
graphs; per-kernel times from fdtd_solver_profile give the roofline;
``e2e`` repeats the run through the C ABI with host buffers (material upload,
a per-step Ez plane snapshot, final field read-back) inside the timed region.
``--impl reference`` times the CPU implementation of the reference kernels
(the FP32 oracle port, bit-identical to them) on all host threads, on the
full grid, with inputs built by the oracle's own readers (no code of this
library runs on that arm).

Multi-GPU (torchrun): every rank runs its own solve (replicas, weak scaling);
value = all ranks' cell-updates / slowest rank's time.
"""
from __future__ import annotations

import argparse
import csv
import gc
import io
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

B_ALG = 97  # bytes per cell-update: 15 state floats read, 9 written, 1-byte class
# algorithmic bytes per cell of each kernel's launch
KERNEL_BYTES = {
    "fused_step": 97,    # H, E^n, E^{n-1}, D^n, D^{n-1} read; H, E, D written; class
    "compact_step": 73,  # H, E^n, R read; H, E, R written; class
    # H, E^n read and written as floats, R as an FP16 residual, one 4-byte scale word per 32 cells, class
    "compact16_step": 61.25,
    "de": 85,            # H, E^n, E^{n-1}, D^n, D^{n-1} read; E, D written; class
    "h": 36,             # H, E read; H written
}
KERNELS = {"single": 0, "two_pass": 1, "compact": 2, "compact16": 3}
# algorithmic bytes per cell-update of a whole step of each state form
FORM_BYTES = {"single": B_ALG, "two_pass": B_ALG, "compact": 73, "compact16": 61.25}
# resident bytes per cell (H double-buffered for the single-pass kernels)
STATE_BYTES = {"single": 73, "two_pass": 61, "compact": 61, "compact16": 55.125}
FORM_STATE = {
    "compact": "H (2 buffers), E (2 slots), R = -a E^{n-1} - 2 tau (D^n - D^{n-1}); D not stored",
    "compact16": "as compact, R stored as the residual R + a E^{n+1} in FP16 with one power-of-two scale "
                 "per 32-cell row segment shared by the three components (11 significant bits for every "
                 "value); FP32 arithmetic; D not stored",
}
# bytes per cell-update of R (read and written) in the compact forms, which
# the strip kernel skips on tile-planes whose classes have no relaxation
R_BYTES = {"compact": 24, "compact16": 12.25}
PRECISION_PROBES = 16
PRECISION_SEED = 2024
METRIC = "cell-updates/s"


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--dims", type=int, nargs=3, default=[512, 512, 400], metavar=("NX", "NY", "NZ"))
    ap.add_argument("--kernel", choices=sorted(KERNELS), default="single")
    ap.add_argument("--scheme", choices=["reference", "corrected"], default="corrected")
    ap.add_argument("--timeskip", type=float, default=0.99, help="dt as a fraction of the Courant limit")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the other forms (compact, 16-bit, batched, served) of the default run")
    ap.add_argument("--workload", choices=["phantom", "batch", "serve"], default="phantom",
                    help="phantom: the 512x512x400 solve (default); batch: 64 uneven solves in one batch; "
                         "serve: a Poisson request stream through the serving loop")
    ap.add_argument("--batch-solves", type=int, default=64, help="solves of the batch workload (the first N)")
    ap.add_argument("--autotune", action="store_true",
                    help="batch workload: choose the z-blocking depth with fdtd_batch_autotune before timing")
    ap.add_argument("--batch-steps", type=int, default=0,
                    help="timed steps of the batch workload (0: until the last solve ends)")
    ap.add_argument("--serve-rate", type=float, default=2.0, help="requests per second (serve)")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="length of the arrival window (serve)")
    ap.add_argument("--serve-policy", choices=["fifo", "sjf"], default="fifo",
                    help="admission order (serve): arrival order or shortest job first")
    ap.add_argument("--serve-max-cells", type=float, default=0.0,
                    help="cap on the cells of the admitted solves (serve; 0: memory budget only)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample length")
    ap.add_argument("--ref-seconds", type=float, default=150.0,
                    help="--impl reference: most seconds of timed CPU steps (fewer steps than --steps if needed)")
    ap.add_argument("--forms-batch-steps", type=int, default=300,
                    help="timed steps of the batched forms in the default run (0: skip them)")
    ap.add_argument("--no-serve-vs-batch", action="store_true",
                    help="skip the served loop against the batch on the same 64 solves (forms.serve_vs_batch)")
    ap.add_argument("--forms-serve-seconds", type=float, default=10.0,
                    help="arrival window of the served form in the default run (20 req/s; 0: skip)")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the probe/DFT/SAR error of the 16-bit-R form against the D form")
    ap.add_argument("--precision-steps", type=int, default=3000, help="steps of the precision comparison")
    return ap.parse_args()


# ---------------------------------------------------------------- workload

def _phantom_module():
    """The input-file writer and phantom generator (pure numpy), loaded on its
    own so that the reference arm runs no code of this library's package."""
    import importlib.util

    name = "fdtd_phantom_inputs"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, ROOT / "fdtd_gb300" / "phantom.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def write_workload_files(nx: int, ny: int, nz: int, tmp: Path):
    """The phantom's class volume plus its input_params and mat_specs files
    (the reference's formats) under tmp.  Returns (codes, number of classes)."""
    ph = _phantom_module()
    codes, mats, cfg = ph.c2_config((nz, ny, nx))
    cfg.env_dir = str(tmp / "pgm")
    cfg.output_dir = str(tmp / "out")
    ph.write_input_params(tmp / "input_params", cfg)
    ph.write_mat_specs(tmp / "mat_specs", mats)
    return codes, len(mats)


def make_workload(nx: int, ny: int, nz: int, tmp: Path, timeskip: float):
    """Phantom codes, class table and Params read back from input_params by
    this library (the GPU arm)."""
    import fdtd_gb300 as fg

    codes, nmats = write_workload_files(nx, ny, nz, tmp)
    p = fg.Params.read(tmp / "input_params")
    p.set_timeskip(timeskip)
    specs = fg.read_specs(tmp / "mat_specs")[:nmats]
    return p, codes, specs


def oracle_inputs(tmp: Path, nmats: int, timeskip: float):
    """The same workload files read by the oracle's restatement of the
    reference's readers: params (initParamsWithPath + timeskip), mat_specs
    records (loadMaterials) and the jz table (setupSources)."""
    from oracle import pyoracle as po

    q = po.params_read(tmp / "input_params", "f32")
    po.set_timeskip(q, timeskip, "f32")
    specs = po.read_specs(tmp / "mat_specs", "f32")[:nmats]
    jz = po.setup_sources(q, "f32")
    return q, specs, jz


def workload_config(args, p) -> dict:
    nx, ny, nz = args.dims
    return {"workload": f"nested-ellipsoid Debye phantom {nx}x{ny}x{nz}, 8 tissue classes + vacuum, "
                        f"900 MHz 3-cell Ez dipole, Mur ABC, dx=1 mm",
            "nx": nx, "ny": ny, "nz": nz, "cells": nx * ny * nz, "scheme": args.scheme, "kernel": args.kernel,
            "sources": [list(s) for s in p.sources], "dt_s": float(p.dt), "timeskip": args.timeskip,
            "l2": f"state {STATE_BYTES[args.kernel] * nx * ny * nz / 1e9:.1f} GB >> 129 MB L2: inputs larger "
                  f"than L2, no flush",
            "b_alg_bytes_per_cell_update": FORM_BYTES[args.kernel]}


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = None

    def __enter__(self):
        try:
            self.out = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if self.proc is None or self.out is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.out.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.out.read())) if len(r) >= 9]
        sm, mx, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                power.append(float(r[3]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def measured_peak_gbs() -> tuple[float, str]:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def committed_traffic(kernel: str, cells: int):
    """DRAM bytes per launch from the committed ncu summary, scaled to cells."""
    f = ROOT / "profiles" / "traffic.json"
    if not f.exists():
        return None
    try:
        rec = json.loads(f.read_text())[kernel]
        return float(rec["dram_bytes_per_cell"]) * cells
    except (KeyError, ValueError):
        return None


# ------------------------------------------------------------- CPU arms

def cpu_port_rate(q, codes, specs, jz, corrected: bool, warmup: int, max_steps: int, seconds: float) -> dict:
    """The FP32 oracle port (bit-identical to the reference kernels run on a
    CPU) on the full grid, OpenMP over (z, y) rows on every host thread the
    process may use: ``warmup`` untimed steps, then timed steps until
    ``max_steps`` or ``seconds`` is reached (at least one).  Returns the rate,
    the threads that ran, the steps timed and the sample's description."""
    from oracle import pyoracle as po

    nx, ny, nz = q.nx, q.ny, q.nz
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    default = [np.full((nz, ny, nx), v, np.float32)
               for v in (q.default_sigma, q.default_eps_s, q.default_eps_i, q.default_tau_d)]
    media.rp = po.setup_mur(q, *default)   # from the default material, as the reference does (fdtd.cu:59,65)
    del default
    cfg = po.make_cfg(q, jz, corrected=corrected)
    threads = po.threads(cfg, "f32")
    st = po.State(nx, ny, nz, np.float32)
    po.run(cfg, media, st, 0, max(1, warmup))
    done, t0 = 0, time.perf_counter()
    while True:
        po.run(cfg, media, st, max(1, warmup) + done, 1)
        done += 1
        el = time.perf_counter() - t0
        if done >= max_steps or el >= seconds:
            break
    cells = nx * ny * nz
    return {"rate": cells * done / el, "threads": threads, "steps": done, "ms_per_step": el / done * 1e3,
            "sample": f"full {nx}x{ny}x{nz} grid, {max(1, warmup)} untimed + {done} timed steps, FP32 port of the "
                      f"reference kernels (bit-identical to them), OpenMP over (z, y) rows on {threads} threads"}


# ------------------------------------------------------------------- arms

def run_reference_arm(args, rank: int, world: int) -> None:
    """The reference's kernels on the host cores: the FP32 oracle port over
    inputs read by the oracle's restatement of the reference's readers (no
    code of this library's package runs here)."""
    if rank != 0:
        return
    nx, ny, nz = args.dims
    with tempfile.TemporaryDirectory() as tmp:
        codes, nmats = write_workload_files(nx, ny, nz, Path(tmp))
        q, specs, jz = oracle_inputs(Path(tmp), nmats, args.timeskip)
    r = cpu_port_rate(q, codes, specs, jz, args.scheme == "corrected", args.warmup, args.steps, args.ref_seconds)
    cfg = {"workload": f"nested-ellipsoid Debye phantom {nx}x{ny}x{nz}, 8 tissue classes + vacuum, "
                       f"900 MHz 3-cell Ez dipole, Mur ABC, dx=1 mm",
           "nx": nx, "ny": ny, "nz": nz, "cells": nx * ny * nz, "scheme": args.scheme, "kernel": "reference",
           "sources": [list(t) for t in q.source_list()], "dt_s": float(q.dt), "timeskip": args.timeskip,
           "b_alg_bytes_per_cell_update": B_ALG}
    line = {"impl": "reference", "metric": METRIC, "value": r["rate"], "unit": "cell-updates/s", "n_gpus": args.gpus,
            "steps": r["steps"], "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg,
            "cpu_baseline": {"value": r["rate"], "unit": "cell-updates/s", "cores": r["threads"], "kind": "port",
                             "sample": r["sample"]},
            "e2e": {"value": r["rate"], "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def precision_probes(codes: np.ndarray, n: int = PRECISION_PROBES, seed: int = PRECISION_SEED):
    """n seeded cells drawn uniformly from the phantom's tissue (class > 0),
    at least 2 cells from every face; (x, y, z) tuples."""
    nz, ny, nx = codes.shape
    inner = np.zeros(codes.shape, bool)
    inner[2:nz - 2, 2:ny - 2, 2:nx - 2] = True
    cand = np.flatnonzero((codes > 0) & inner)
    pick = np.random.default_rng(seed).choice(cand, size=n, replace=False)
    z, rem = np.divmod(pick, ny * nx)
    y, x = np.divmod(rem, nx)
    return [(int(a), int(b), int(c)) for a, b, c in zip(x, y, z)]


C3_FIXTURE = ROOT / "tests" / "golden" / "c3_fp64.npz"


def c3_fixture(p, codes, specs, steps: int, scheme: str):
    """The FP64 oracle's record of this workload (tests/golden/c3_fp64.npz),
    when it describes exactly these inputs, else None."""
    import hashlib

    if not C3_FIXTURE.exists() or scheme != "corrected":
        return None
    f = np.load(C3_FIXTURE)
    same = (tuple(int(v) for v in f["shape"]) == codes.shape and int(f["steps"]) == steps
            and np.float32(p.dt) == f["dt"] and np.array_equal(f["specs"], specs)
            and str(f["codes_sha256"]) == hashlib.sha256(codes.tobytes()).hexdigest())
    return f if same else None


def precision_check(p, codes, specs, dev: int, steps: int, scheme: str) -> dict:
    """Error of the 16-bit-R compact form, the 32-bit compact form and the D
    form against the FP64 oracle, corrected scheme, `steps` steps: E series at
    16 seeded probe points inside the phantom (relative L2 per probe over the
    3 components and all steps), the running DFT |E| at the source's 900 MHz
    over 32 planes through the source (on every 4th cell in x and y, as the
    oracle's record holds it), and the peak spectral SAR over those planes.
    The FP64 record comes from tests/golden/make_c3_fixture.py; without one for
    this workload the D form on the GPU stands in for it."""
    import fdtd_gb300 as fg

    nz = codes.shape[0]
    fx = c3_fixture(p, codes, specs, steps, scheme)
    probes = [tuple(int(v) for v in r) for r in fx["probes"]] if fx is not None else precision_probes(codes)
    freq = float(p.waveFrequency) * float(p.pulseModulationFrequency)
    z0, nplanes = max(0, nz // 2 - 16), min(32, nz)
    sub = int(fx["dft_sub"]) if fx is not None else 1

    def run(kernel):
        s = fg.Solver(p, codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel, device=dev)
        s.set_probes(probes, capacity=steps)
        s.set_dft(freq, stride=5, z0=z0, nplanes=nplanes)
        s.run(steps)
        s.synchronize()
        series = s.probes().astype(np.float64)
        e2 = None
        for comp in range(3):
            a = s.dft(comp)
            e2 = np.abs(a) ** 2 if e2 is None else e2 + np.abs(a) ** 2
        sar, cell = s.peak_sar()
        s.close()
        return series, np.sqrt(e2)[:, ::sub, ::sub], sar, cell

    if fx is not None:
        pc = fx["peak_sar_cell"]
        ny, nx = codes.shape[1:]
        ref = (fx["series"].astype(np.float64), fx["dft_abs_e_sub"].astype(np.float64), float(fx["peak_sar"]),
               int((pc[2] * ny + pc[1]) * nx + pc[0]))
        what = ("FP64 CPU oracle (tests/golden/c3_fp64.npz: same phantom, corrected scheme, dt 0.99 of the "
                "Courant limit)")
        forms = (("compact16", fg.KERNEL_COMPACT_R16), ("compact", fg.KERNEL_COMPACT), ("d_form", fg.KERNEL_SINGLE_PASS))
    else:
        ref = run(fg.KERNEL_SINGLE_PASS)
        what = "FP32 D form on the GPU (no FP64 record of this workload)"
        forms = (("compact16", fg.KERNEL_COMPACT_R16), ("compact", fg.KERNEL_COMPACT))
    out = {"reference": what, "steps": steps, "probes": probes, "dft_hz": freq, "dft_planes": [z0, z0 + nplanes],
           "dft_cells": f"every {sub}th cell in x and y" if sub > 1 else "all"}
    for name, kernel in forms:
        series, amp, sar, cell = run(kernel)
        per = [float(np.linalg.norm(series[:, j] - ref[0][:, j]) / max(np.linalg.norm(ref[0][:, j]), 1e-300))
               for j in range(len(probes))]
        out[name] = {"probe_rel_l2_max": max(per), "probe_rel_l2_median": float(np.median(per)),
                     "probe_rel_l2": per,
                     "dft_abs_e_rel_l2": float(np.linalg.norm(amp - ref[1]) / np.linalg.norm(ref[1])),
                     "peak_sar_rel": float(abs(sar - ref[2]) / ref[2]), "peak_sar_same_cell": cell == ref[3]}
    return out


def ref_cuda_leg(q, codes, specs, jz, dev: int, steps: int = 300, warmup: int = 6) -> dict | None:
    """The reference's own CUDA kernels (fdtd_calculations.cu compiled for
    sm_103a with its Makefile's nvcc defaults, run from the cubin with its
    launch grid and slot rotation, output gated) on this workload and GPU,
    outside the timed region.  Steps stay below 512 (the reference's dJz
    table); None where the cubin was not built."""
    from oracle import pyoracle as po

    if not po.ref_gpu_available():
        return None
    nx, ny, nz = q.nx, q.ny, q.nz
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    default = [np.full((nz, ny, nx), v, np.float32)
               for v in (q.default_sigma, q.default_eps_s, q.default_eps_i, q.default_tau_d)]
    media.rp = po.setup_mur(q, *default)
    del default
    with ClockSampler(dev) as clk:
        ms = po.ref_gpu_run(po.make_cfg(q, jz), media, steps, warmup=warmup)
    cells = nx * ny * nz
    return {"value": cells * steps / (ms / 1e3), "unit": "cell-updates/s", "ms_per_step": ms / steps,
            "steps": steps, "warmup": warmup, "clocks": clk.summary(),
            "what": "the reference's fdtd_calculations.cu kernels (nvcc defaults, sm_103a) with its launch grid "
                    "(ceil(nx/128) x ny x nz blocks of 128) and slot rotation, reference scheme, same workload, "
                    "same GPU, CUDA events around the steps"}


def run_gb300_arm(args, rank: int, local_rank: int, world: int, dist) -> None:
    import torch

    import fdtd_gb300 as fg
    from fdtd_gb300 import replicas

    torch.cuda.set_device(local_rank)
    nx, ny, nz = args.dims
    cells = nx * ny * nz
    kernel = KERNELS[args.kernel]
    scheme = fg.SCHEME_REFERENCE if args.scheme == "reference" else fg.SCHEME_CORRECTED
    tmp = tempfile.TemporaryDirectory()
    p, codes, specs = make_workload(nx, ny, nz, Path(tmp.name), args.timeskip)

    # ---- device-resident throughput (value)
    s = fg.Solver(p, codes, specs, scheme=scheme, kernel=kernel, device=local_rank)
    stream = torch.cuda.ExternalStream(s.stream)
    s.run(args.warmup)
    s.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        replicas.barrier(dist)
        torch.cuda.synchronize()
        start.record(stream)
        s.run(args.steps)
        end.record(stream)
        s.synchronize()
        torch.cuda.synchronize()
        replicas.barrier(dist)
    seconds = start.elapsed_time(end) / 1e3
    total_cells, tmax = replicas.aggregate(cells * args.steps, seconds, dist, device=f"cuda:{local_rank}")
    clocks = clk.summary()
    prof = s.profile(min(args.steps, 20))
    kernels_per_step = len(prof)
    s.close()

    # ---- end to end through the C ABI with host buffers (e2e), right after
    # the device-resident run of the same workload
    e2e = None
    if not args.no_e2e:
        srcz = p.sources[0][2] if p.sources else nz // 2
        plane_bytes = 4 * nx * ny
        got = []
        # the caller's host result buffer exists before the timed region, as
        # its host inputs do (its pages already touched)
        final = np.zeros((nz, ny, nx), np.float32)
        final.fill(1.0)
        gc.collect()  # no collection of earlier garbage inside the timed region
        torch.cuda.synchronize()
        replicas.barrier(dist)
        t0 = time.perf_counter()
        s2 = fg.Solver(p, codes, specs, scheme=scheme, kernel=kernel, device=local_rank)
        s2.set_snapshots(every=1, fields=("ez",), z0=srcz, nplanes=1, callback=lambda st, n, a: got.append(st))
        s2.run(args.steps)
        s2.flush_snapshots()
        s2.field("ez", out=final)
        s2.close()
        t1 = time.perf_counter()
        replicas.barrier(dist)
        assert len(got) == args.steps and final.shape == (nz, ny, nx)
        # copied from the host: the class volume, the plan's 256-entry class
        # table (32 B each) and its 65536-entry source table; the Mur slabs
        # of the default material are filled on the device
        h2d = codes.nbytes + 256 * 32 + 4 * 65536
        d2h = plane_bytes * args.steps + final.nbytes
        e_cells, e_t = replicas.aggregate(cells * args.steps, t1 - t0, dist, device=f"cuda:{local_rank}")
        e2e = {"value": e_cells / e_t, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d / args.steps,
               "d2h_bytes_per_step": d2h / args.steps,
               "includes": "solver create (material + plan upload), per-step Ez plane D2H through the pinned "
                           "snapshot ring, final Ez volume read-back into a host buffer allocated before the "
                           "timed region, destroy"}

    # ---- the compact forms on the same workload (reported beside the D
    # form; same metric, same timing rules, their own clock records)
    forms = {}
    if args.kernel == "single" and not args.no_forms:
        for fname in ("compact", "compact16"):
            c = fg.Solver(p, codes, specs, scheme=scheme, kernel=KERNELS[fname], device=local_rank)
            cstream = torch.cuda.ExternalStream(c.stream)
            c.run(args.warmup)
            c.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with ClockSampler(local_rank) as cclk:
                replicas.barrier(dist)
                torch.cuda.synchronize()
                a.record(cstream)
                c.run(args.steps)
                b.record(cstream)
                c.synchronize()
                torch.cuda.synchronize()
                replicas.barrier(dist)
            c_cells, c_t = replicas.aggregate(cells * args.steps, a.elapsed_time(b) / 1e3, dist,
                                              device=f"cuda:{local_rank}")
            cprof = c.profile(min(args.steps, 20))
            memless = c.memless_fraction
            c.close()
            cmain = max(cprof, key=cprof.get)
            # R is neither read nor written on tile-planes without Debye memory
            eff = KERNEL_BYTES.get(cmain, 0) - R_BYTES[fname] * memless
            forms[fname] = {
                "value": c_cells / c_t, "unit": "cell-updates/s", "ms_per_step": c_t / args.steps * 1e3,
                "state": FORM_STATE[fname], "b_alg_bytes_per_cell_update": FORM_BYTES[fname],
                "memless_fraction": memless, "b_alg_effective": eff, "kernel_ms": cprof,
                "roofline_kernel": cmain,
                "roofline_achieved_gbs": eff * cells / (cprof[cmain] / 1e3) / 1e9,
                "roofline_achieved_gbs_dense_basis": KERNEL_BYTES.get(cmain, 0) * cells / (cprof[cmain] / 1e3) / 1e9,
                "roofline_traffic": committed_traffic(cmain, cells),
                "gpu_launches": len(cprof) * args.steps, "clocks": cclk.summary()}
        if not args.no_precision:
            forms["compact16"]["precision"] = precision_check(p, codes, specs, local_rank, args.precision_steps,
                                                              args.scheme)
    # ---- the batched (64 uneven solves, both storage forms) and served
    # (request stream, 16-bit form) forms, N = 1 only
    if args.kernel == "single" and not args.no_forms and world == 1 and args.forms_batch_steps > 0:
        reqs = batch_requests(64)
        btmp = tempfile.TemporaryDirectory()
        binputs = _request_inputs(reqs, Path(btmp.name))
        forms["batch"] = {k: batch_form(k, reqs, binputs, args.warmup, args.forms_batch_steps, True)
                          for k in ("compact", "compact16")}
        if not args.no_serve_vs_batch:
            forms["serve_vs_batch"] = serve_vs_batch("compact16", reqs, binputs)
        del binputs
        btmp.cleanup()
    if args.kernel == "single" and not args.no_forms and world == 1 and args.forms_serve_seconds > 0:
        forms["serve"] = serve_form("compact16", 20.0, args.forms_serve_seconds)

    # ---- CPU baseline and the reference's CUDA kernels (rank 0, N = 1 only;
    # inputs read by the oracle's restatement of the reference's readers)
    cpu = ref_cuda = None
    if rank == 0 and world == 1 and not args.no_cpu:
        q, ospecs, jz = oracle_inputs(Path(tmp.name), len(specs), args.timeskip)
        r = cpu_port_rate(q, codes, ospecs, jz, args.scheme == "corrected", 2, 10 ** 6, args.cpu_seconds)
        cpu = {"value": r["rate"], "unit": "cell-updates/s", "cores": r["threads"], "kind": "port",
               "sample": r["sample"]}
        ref_cuda = ref_cuda_leg(q, codes, ospecs, jz, local_rank)
        if ref_cuda is not None:
            ref_cuda["speedup_value_vs_ref_cuda"] = (total_cells / tmax) / ref_cuda["value"]
    tmp.cleanup()

    if rank != 0:
        return
    peak, peak_kind = measured_peak_gbs()
    main = max(prof, key=prof.get)
    main_ms = prof[main]
    main_bytes = KERNEL_BYTES.get(main, B_ALG)
    achieved = main_bytes * cells / (main_ms / 1e3) / 1e9
    step_ms = sum(prof.values())
    line = {
        "metric": METRIC, "value": total_cells / tmax, "unit": "cell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tmax / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, p),
        "roofline": {"bound": "hbm", "kernel": main, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": committed_traffic(main, cells),
                     "algorithmic_bytes_per_launch": main_bytes * cells, "avg_launch_ms": main_ms,
                     "step_hbm_frac": FORM_BYTES[args.kernel] * cells / (step_ms / 1e3) / 1e9 / peak},
        "kernel_ms": prof,
        "gpu_launches": kernels_per_step * args.steps,
        "clocks": clocks,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "ref_cuda_baseline": ref_cuda,
    }
    if forms:
        for f in forms.values():
            if "roofline_achieved_gbs" in f:
                f["roofline_frac"] = f["roofline_achieved_gbs"] / peak
                f["roofline_frac_dense_basis"] = f["roofline_achieved_gbs_dense_basis"] / peak
        line["forms"] = forms
    print(json.dumps(line), flush=True)


# ------------------------------------------------------- batched / served

FORM_NAMES = {"single": "D form", "two_pass": "D form", "compact": "compact form (H, E, R)",
              "compact16": "compact form with 16-bit R (H, E, R16)"}


def _request_inputs(reqs, root: Path, threads: int = 8) -> dict:
    """Inputs of each request (input_params + mat_specs + class volume), built
    in parallel before the clock starts: they arrive with the requests."""
    from concurrent.futures import ThreadPoolExecutor

    from fdtd_gb300 import serve as sv

    def one(r):
        return r.rid, sv.build_inputs(r, root / str(r.rid))

    with ThreadPoolExecutor(threads) as ex:
        return dict(ex.map(one, reqs))


def batch_requests(n: int = 64):
    """The 64-solve batch: dims log-uniform 48-256 per axis, 1-4 Debye
    ellipsoids each, source U[0.3, 3] GHz, steps U[500, 3000] (seeded)."""
    from fdtd_gb300 import serve as sv

    rng = np.random.default_rng(1234)
    reqs = []
    for rid in range(64):
        dims = tuple(int(round(math.exp(rng.uniform(math.log(48), math.log(256))))) for _ in range(3))
        reqs.append(sv.Request(rid, 0.0, dims, float(rng.uniform(3e8, 3e9)), int(rng.integers(500, 3001)),
                               int(rng.integers(1 << 30))))
    return reqs[:max(1, min(64, n))]


def batch_form(kernel_name: str, reqs, inputs: dict, warmup: int, steps: int, autotune: bool) -> dict:
    """All solves in one batch of the given form: warm-up steps, the optional
    autotuner (its trial steps are real steps, before the timed region), then
    `steps` timed steps (0: until the last solve ends).  value = cell-updates
    of all solves in the timed steps / device time of those steps."""
    import torch

    import fdtd_gb300 as fg

    b = fg.Batch(0, KERNELS[kernel_name])
    ids = []
    for r in reqs:
        p, codes, specs, src = inputs[r.rid]
        ids.append(b.add(p, codes, specs, r.steps, scheme=fg.SCHEME_CORRECTED))
    warm = max(3, warmup)
    b.run(warm)
    b.synchronize()
    zchunk = b.autotune() if autotune else 0
    pre = [b.steps(i) for i in ids]
    stream = torch.cuda.ExternalStream(b.stream)
    a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    to_run = max(r.steps - d for r, d in zip(reqs, pre))
    if steps > 0:
        to_run = min(to_run, steps)
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        a.record(stream)
        b.run(to_run)
        e.record(stream)
        b.synchronize()
        torch.cuda.synchronize()
    seconds = a.elapsed_time(e) / 1e3
    post = [b.steps(i) for i in ids]
    assert all(q == min(r.steps, d + to_run) for q, d, r in zip(post, pre, reqs))
    cells = [r.dims[0] * r.dims[1] * r.dims[2] for r in reqs]
    updates = sum(c * (q - d) for c, q, d in zip(cells, post, pre))
    peak, peak_kind = measured_peak_gbs()
    bpc = FORM_BYTES[kernel_name]
    out = {"value": updates / seconds, "unit": "cell-updates/s", "steps": to_run, "warmup": warm,
           "ms_per_step": seconds / to_run * 1e3, "form": FORM_NAMES[kernel_name], "solves": len(reqs),
           "cells_total": sum(cells), "state_bytes": b.bytes, "cell_updates": updates,
           "z_chunk_limit": zchunk or "default", "tuning": b.tuning(),
           "autotune": "fdtd_batch_autotune before timing (its trial steps are excluded)" if autotune else "off",
           "roofline": {"bound": "hbm", "kernel": "batch step (all kernels)", "achieved": bpc * updates / seconds / 1e9,
                        "peak": peak, "unit": "GB/s", "frac": bpc * updates / seconds / 1e9 / peak,
                        "peak_kind": peak_kind, "algorithmic_bytes_per_cell_update": bpc},
           "gpu_launches": 3 * to_run, "clocks": clk.summary()}
    b.close()
    return out


def serve_vs_batch(kernel_name: str, reqs, inputs: dict) -> dict:
    """The served loop against the batch on the same solves, both to the
    last solve's end: the 64 batch solves arrive at once (the served form at
    saturation), 25-step chunks, an Ez snapshot every 250 steps; the batch
    runs them in one batch with no autotuning.  Rates are all cell-updates
    over the wall time from the first arrival (served) and over the device
    time of the steps after 3 warm-up steps (batched)."""
    import fdtd_gb300 as fg
    from fdtd_gb300 import serve as sv

    batch = batch_form(kernel_name, reqs, inputs, 3, 0, False)
    reqs0 = [sv.Request(r.rid, 0.0, r.dims, r.frequency, r.steps, r.seed) for r in reqs]
    with ClockSampler(0) as clk:
        res = sv.serve(reqs0, budget_bytes=150 * 10 ** 9, chunk=25, snapshot_every=250, scheme=fg.SCHEME_CORRECTED,
                       inputs=dict(inputs), kernel=KERNELS[kernel_name])
    summ = res.summary()
    return {"form": FORM_NAMES[kernel_name], "solves": len(reqs),
            "batched": {"value": batch["value"], "ms_per_step": batch["ms_per_step"], "steps": batch["steps"],
                        "clocks": batch["clocks"]},
            "served": {"value": summ["cell_updates_per_s"], "wall_s": summ["wall_s"],
                       "gpu_busy_fraction": summ["gpu_busy_fraction"], "completed": summ["completed"],
                       "p50_ms": summ["p50_ms"], "p99_ms": summ["p99_ms"], "clocks": clk.summary()},
            "served_over_batched": summ["cell_updates_per_s"] / batch["value"]}


def serve_form(kernel_name: str, rate: float, seconds: float, policy: str = "fifo", max_cells: float = 0.0,
               inputs_threads: int = 8) -> dict:
    """A Poisson request stream (dims log-uniform 64-384 per axis, Debye
    ellipsoids, source U[0.3,3] GHz, steps U[500,4000]) through the serving
    loop: admission against a 150 GB budget, continuous batching, Ez
    snapshot every 250 steps streamed to the host.  Latency is arrival to
    completion; request inputs are built before the clock starts (they arrive
    with the requests)."""
    import fdtd_gb300 as fg
    from fdtd_gb300 import serve as sv

    reqs = sv.poisson_stream(rate, seconds, seed=7, dims=(64, 384), steps=(500, 4000))
    tmp = tempfile.TemporaryDirectory()
    inputs = _request_inputs(reqs, Path(tmp.name), inputs_threads)
    snaps = []
    with ClockSampler(0) as clk:
        res = sv.serve(reqs, budget_bytes=150 * 10 ** 9, chunk=25, snapshot_every=250, scheme=fg.SCHEME_CORRECTED,
                       inputs=inputs, on_snapshot=lambda r, step, plane: snaps.append(plane.nbytes),
                       kernel=KERNELS[kernel_name], policy=policy, max_active_cells=max_cells or None)
    tmp.cleanup()
    summ = res.summary()
    return {"value": summ["cell_updates_per_s"], "unit": "cell-updates/s", "form": FORM_NAMES[kernel_name],
            "stream": f"Poisson {rate} req/s for {seconds} s, dims log-uniform 64-384, steps U[500,4000], 150 GB "
                      f"budget, Ez snapshot every 250 steps (pinned copies on the batch stream), corrected scheme",
            "requests": len(reqs), "policy": policy, "max_active_cells": max_cells or "memory budget only",
            "serve": {**summ, "snapshot_bytes": int(sum(snaps)), "snapshots": len(snaps)},
            "clocks": clk.summary()}


def run_batch_workload(args) -> None:
    """--workload batch: the 64-solve batch in the --kernel form, one line."""
    reqs = batch_requests(args.batch_solves)
    tmp = tempfile.TemporaryDirectory()
    inputs = _request_inputs(reqs, Path(tmp.name))
    kname = args.kernel if args.kernel in ("compact", "compact16") else "single"
    f = batch_form(kname, reqs, inputs, args.warmup, args.batch_steps, args.autotune)
    tmp.cleanup()
    line = {
        "metric": METRIC, "value": f["value"], "unit": "cell-updates/s", "n_gpus": 1, "steps": f["steps"],
        "warmup": f["warmup"], "ms_per_step": f["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batch of {len(reqs)} solves, dims log-uniform 48-256 per axis, 1-4 Debye "
                               f"ellipsoids, source U[0.3,3] GHz, steps U[500,3000], corrected scheme, {f['form']}",
                   **{k: f[k] for k in ("solves", "cells_total", "state_bytes", "cell_updates", "z_chunk_limit", "tuning",
                                        "autotune")}, "l2": "state >> 129 MB L2: no flush"},
        "roofline": {**f["roofline"], "traffic": None}, "gpu_launches": f["gpu_launches"], "clocks": f["clocks"],
        "e2e": None, "cpu_baseline": None}
    print(json.dumps(line), flush=True)


def run_serve_workload(args) -> None:
    """--workload serve: the request stream in the --kernel form, one line."""
    kname = args.kernel if args.kernel in ("compact", "compact16") else "single"
    f = serve_form(kname, args.serve_rate, args.serve_seconds, args.serve_policy, args.serve_max_cells)
    line = {"metric": "served cell-updates/s and latency", "value": f["value"], "unit": "cell-updates/s",
            "n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"{f['stream']}, {f['form']}", "requests": f["requests"], "policy": f["policy"],
                       "max_active_cells": f["max_active_cells"]},
            "serve": f["serve"], "clocks": f["clocks"]}
    print(json.dumps(line), flush=True)


def main() -> None:
    args = parse_args()
    if args.impl == "gb300" and args.workload != "phantom":
        import torch

        torch.cuda.set_device(0)
        (run_batch_workload if args.workload == "batch" else run_serve_workload)(args)
        return
    if args.impl == "reference":
        # rank 0 alone runs the CPU arm; other ranks exit without work (no
        # process group: the arm has no exchange)
        run_reference_arm(args, int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)))
        return
    from fdtd_gb300 import replicas

    rank, local_rank, world = replicas.dist_env()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td

        torch.cuda.set_device(local_rank)
        td.init_process_group("nccl")
        dist = td
    try:
        run_gb300_arm(args, rank, local_rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
