"""Serving loop: solve requests admitted into one running batch.

Requests (grid, seeded phantom, source frequency, step count) arrive as a
Poisson stream.  Between chunks of batched steps the loop admits queued
requests (in arrival order, or shortest job first) while their device state
fits the memory budget and, optionally, their cells fit a cap,
streams a snapshot (the Ez plane through the source) of every solve whose step
count reached a multiple of the snapshot period, and retires finished solves,
freeing their memory for the queue.  Work of all admitted solves overlaps on
the device in the same batched launches (continuous batching).  Latency is
arrival to completion.  No reference counterpart (the reference runs one
grid per process).
"""
from __future__ import annotations

import math
import tempfile
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import KERNEL_SINGLE_PASS, SCHEME_CORRECTED, Batch, Params
from . import phantom as ph


@dataclass
class Request:
    rid: int
    arrival: float            # seconds after the stream starts
    dims: tuple[int, int, int]
    frequency: float
    steps: int
    seed: int
    # filled by the server
    admitted: float = math.nan
    done: float = math.nan
    snapshots: list = field(default_factory=list)   # (step, Ez plane)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def poisson_stream(rate: float, duration: float, seed: int = 0, dims=(64, 384), steps=(500, 4000),
                   freq=(3.0e8, 3.0e9)) -> list[Request]:
    """Arrivals of a Poisson process; dims log-uniform per axis, steps and
    source frequency uniform."""
    rng = np.random.default_rng(seed)
    out, t, rid = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            return out
        d = tuple(int(round(math.exp(rng.uniform(math.log(dims[0]), math.log(dims[1]))))) for _ in range(3))
        out.append(Request(rid, t, d, float(rng.uniform(*freq)), int(rng.integers(steps[0], steps[1] + 1)),
                           int(rng.integers(1 << 30))))
        rid += 1


def build_inputs(req: Request, root: Path):
    """Params, class volume and class table of one request (the reference's
    formats: input_params + mat_specs; 1-4 Debye ellipsoids in vacuum)."""
    nx, ny, nz = req.dims
    rng = np.random.default_rng(req.seed)
    nshell = int(rng.integers(1, 5))
    semi = min(nx, ny, nz) / 2 - 3
    codes, mats, outer = ph.ellipsoid_phantom((nz, ny, nx), n_shells=nshell, seed=req.seed,
                                              semi_min=0.25 * semi, semi_max=0.8 * semi)
    epw = max(10, int(round(3.0e8 / (req.frequency * 1.0e-3))))   # dx close to 1 mm
    src = (max(1, nx // 8), ny // 2, nz // 2)
    cfg = ph.Config(nx, ny, nz, req.steps, wave_frequency=req.frequency, elements_per_wavelength=epw,
                    pulse_width=0.5, pulse_modulation_frequency=1.0, sources=[src])
    root.mkdir(parents=True, exist_ok=True)
    ph.write_input_params(root / "input_params", cfg)
    ph.write_mat_specs(root / "mat_specs", mats)
    p = Params.read(root / "input_params")
    p.set_timeskip(0.99)
    from . import read_specs
    specs = read_specs(root / "mat_specs")[: len(mats)]
    return p, codes, specs, src


@dataclass
class ServeResult:
    requests: list
    wall: float
    cell_updates: float

    def summary(self) -> dict:
        lat = np.array([r.latency for r in self.requests if not math.isnan(r.done)])
        return {"completed": int(lat.size), "requested": len(self.requests),
                "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
                "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None,
                "cell_updates_per_s": self.cell_updates / self.wall if self.wall > 0 else None,
                "wall_s": self.wall}


def work(req: Request) -> float:
    """Cell-updates of a request."""
    return float(req.dims[0]) * req.dims[1] * req.dims[2] * req.steps


def order_queue(queue: list[Request], policy: str) -> None:
    """Admission order, in place: "fifo" keeps arrival order, "sjf" puts the
    request with the least work first (ties by arrival)."""
    if policy == "sjf":
        queue.sort(key=lambda r: (work(r), r.arrival))
    elif policy != "fifo":
        raise ValueError(f"unknown policy {policy!r}")


def serve(requests: list[Request], budget_bytes: int, chunk: int = 25, snapshot_every: int = 250,
          scheme: int = SCHEME_CORRECTED, device: int = 0, clock=time.perf_counter,
          on_snapshot=None, inputs: dict | None = None, kernel: int = KERNEL_SINGLE_PASS,
          policy: str = "fifo", max_active_cells: float | None = None) -> ServeResult:
    """Runs the request stream to completion in real time.  chunk must
    divide snapshot_every so snapshots land on exact step counts.  inputs
    (optional) maps request ids to build_inputs results that arrive with the
    requests; missing ones are built at admission.  kernel selects the state
    form of every solve (KERNEL_SINGLE_PASS, KERNEL_COMPACT or
    KERNEL_COMPACT_R16).  policy: the admission order ("fifo" or "sjf", see order_queue).  max_active_cells
    (optional) caps the cells of the admitted solves: the batched launch
    needs only enough of them to fill the GPU, and admitting more only shares
    it among more requests, which lengthens every one; a request is admitted
    alone when nothing runs, whatever its size."""
    assert snapshot_every % chunk == 0
    order_queue([], policy)  # rejects an unknown policy before any work
    pending = sorted(requests, key=lambda r: r.arrival)
    queue: list[Request] = []
    active: dict[int, tuple[Request, int, int, Params]] = {}  # sid -> (req, steps done, snapshot z, params)
    batch = Batch(device, kernel)
    tmp = tempfile.TemporaryDirectory()
    cell_updates = 0.0
    active_cells = 0.0
    t0 = clock()
    try:
        while pending or queue or active:
            now = clock() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.pop(0))
            # admit in policy order while the head fits the budget and the cap
            order_queue(queue, policy)
            while queue:
                req = queue[0]
                need = batch.need_bytes(*req.dims)
                if need > budget_bytes:
                    queue.pop(0)  # can never fit: drop (done stays NaN)
                    continue
                if batch.bytes + need > budget_bytes:
                    break
                cells = float(req.dims[0]) * req.dims[1] * req.dims[2]
                if max_active_cells is not None and active and active_cells + cells > max_active_cells:
                    break
                queue.pop(0)
                if inputs is not None and req.rid in inputs:
                    p, codes, specs, src = inputs.pop(req.rid)
                else:
                    p, codes, specs, src = build_inputs(req, Path(tmp.name) / str(req.rid))
                sid = batch.add(p, codes, specs, req.steps, scheme=scheme)
                req.admitted = clock() - t0
                active[sid] = (req, 0, src[2], p)
                active_cells += cells
            if not active:
                if pending:  # idle until the next arrival
                    time.sleep(max(0.0, min(0.05, pending[0].arrival - (clock() - t0))))
                continue
            batch.run(chunk)
            batch.synchronize()
            finished = []
            for sid, (req, done, sz, p) in list(active.items()):
                adv = min(chunk, req.steps - done)
                cell_updates += float(adv) * req.dims[0] * req.dims[1] * req.dims[2]
                done += adv
                if done % snapshot_every == 0 or done == req.steps:
                    plane = batch.field(sid, "ez", z0=sz, nplanes=1)[0]
                    req.snapshots.append(done)
                    if on_snapshot is not None:
                        on_snapshot(req, done, plane)
                active[sid] = (req, done, sz, p)
                if done >= req.steps:
                    finished.append(sid)
            for sid in finished:
                req = active.pop(sid)[0]
                active_cells -= float(req.dims[0]) * req.dims[1] * req.dims[2]
                req.done = clock() - t0
                if on_snapshot is not None and hasattr(on_snapshot, "final"):
                    on_snapshot.final(req, batch, sid)
                batch.remove(sid)
    finally:
        wall = clock() - t0
        batch.close()
        tmp.cleanup()
    return ServeResult(requests, wall, cell_updates)
