"""Serving loop: solve requests admitted into one running batch.

Requests (grid, seeded phantom, source frequency, step count) arrive as a
Poisson stream.  Between chunks of batched steps the loop admits queued
requests (in arrival order, or shortest job first) while their device state
fits the memory budget and, optionally, their cells fit a cap, queues a
snapshot copy (the Ez plane through the source) of every solve whose step
count reaches a multiple of the snapshot period, and retires finished solves,
freeing their memory for the queue.  Work of all admitted solves overlaps on
the device in the same batched launches (continuous batching).

The loop never drains the GPU to do this bookkeeping: it keeps up to
``inflight`` chunks queued, admits new solves while earlier chunks run (their
uploads go on a side stream), copies snapshots into page-locked buffers on
the batch stream and hands them over once their ticket reports done, and
learns that a request finished from a marker queued after its last chunk.
Requests can be cancelled from the host (``ServeControl.cancel``) or carry a
deadline; either ends the request without touching the other solves, and a
failed request never takes the loop down with it (the reference stops the
whole process on any error, utils.h:5-13).  Latency is arrival to
completion.  No reference counterpart (the reference runs one grid per
process).
"""
from __future__ import annotations

import math
import tempfile
import threading
import time
from collections import deque
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import KERNEL_SINGLE_PASS, SCHEME_CORRECTED, Batch, FdtdError, Params, PinnedBuffer
from . import phantom as ph


@dataclass
class Request:
    rid: int
    arrival: float            # seconds after the stream starts
    dims: tuple[int, int, int]
    frequency: float
    steps: int
    seed: int
    deadline: float = math.inf  # seconds after arrival by which it must finish (else it is ended)
    # filled by the server
    admitted: float = math.nan
    done: float = math.nan
    status: str = "pending"     # done, cancelled, deadline, rejected (never fits the budget), failed
    error: str = ""             # why it failed
    snapshots: list = field(default_factory=list)   # steps at which a snapshot was delivered

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
    gpu_busy_ms: float = 0.0   # GPU time of the batched steps
    gpu_span_ms: float = 0.0   # from the first batched step's start to the last one's end

    def summary(self) -> dict:
        lat = np.array([r.latency for r in self.requests if r.status == "done"])
        count = {k: sum(r.status == k for r in self.requests)
                 for k in ("cancelled", "deadline", "rejected", "failed")}
        return {"completed": int(lat.size), "requested": len(self.requests), **count,
                "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
                "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None,
                "cell_updates_per_s": self.cell_updates / self.wall if self.wall > 0 else None,
                "wall_s": self.wall,
                "gpu_busy_fraction": self.gpu_busy_ms / self.gpu_span_ms if self.gpu_span_ms > 0 else None,
                "gpu_busy_s": self.gpu_busy_ms / 1e3}


class ServeControl:
    """Host-side control of a running serve(): cancel(rid) ends a request
    (queued or running) at the loop's next turn; thread-safe."""

    def __init__(self):
        self._lock = threading.Lock()
        self._cancel: set[int] = set()

    def cancel(self, rid: int) -> None:
        with self._lock:
            self._cancel.add(rid)

    def take(self) -> set[int]:
        with self._lock:
            out, self._cancel = self._cancel, set()
        return out


class _Buffers:
    """Page-locked snapshot buffers, reused by size."""

    def __init__(self):
        self.free: dict[int, list[PinnedBuffer]] = {}
        self.all: list[PinnedBuffer] = []

    def get(self, n: int) -> PinnedBuffer:
        lst = self.free.get(n)
        if lst:
            return lst.pop()
        b = PinnedBuffer(n)
        self.all.append(b)
        return b

    def put(self, n: int, b: PinnedBuffer) -> None:
        self.free.setdefault(n, []).append(b)

    def close(self) -> None:
        for b in self.all:
            b.close()
        self.all.clear()
        self.free.clear()


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
          policy: str = "fifo", max_active_cells: float | None = None, control: ServeControl | None = None,
          inflight: int = 2, admit_per_turn: int = 4) -> ServeResult:
    """Runs the request stream to completion in real time.  chunk must
    divide snapshot_every so snapshots land on exact step counts.  inputs
    (optional) maps request ids to build_inputs results that arrive with the
    requests; missing ones are built at admission.  kernel selects the state
    form of every solve (KERNEL_SINGLE_PASS, KERNEL_COMPACT or
    KERNEL_COMPACT_R16).  policy: the admission order ("fifo" or "sjf", see
    order_queue).  max_active_cells (optional) caps the cells of the admitted
    solves: the batched launch needs only enough of them to fill the GPU, and
    admitting more only shares it among more requests, which lengthens every
    one; a request is admitted alone when nothing runs, whatever its size.
    on_snapshot(req, step, plane) receives each snapshot (a copy the callee
    may keep).  control (optional) cancels requests from the host; a request
    whose deadline passes is ended the same way.  inflight: batched chunks
    queued ahead of the host.  admit_per_turn: requests admitted per turn of
    the loop once solves run, so that building and uploading new solves
    overlaps the queued chunks instead of holding the next chunk back (when
    nothing runs, one request is admitted and stepped at once)."""
    assert snapshot_every % chunk == 0 and inflight >= 1
    order_queue([], policy)  # rejects an unknown policy before any work
    pending = deque(sorted(requests, key=lambda r: r.arrival))
    queue: list[Request] = []
    active: dict[int, list] = {}   # sid -> [req, steps queued, snapshot z, params]
    chunks: deque[int] = deque()   # tickets of the queued chunks (oldest first)
    snaps: list[tuple] = []        # (ticket, req, step, buffer, n, shape) of queued snapshot copies
    finishing: list[tuple] = []    # (ticket, req) of requests whose last chunk is queued
    bufs = _Buffers()
    batch = Batch(device, kernel)
    batch.set_timing(True)
    tmp = tempfile.TemporaryDirectory()
    cell_updates = 0.0
    active_cells = 0.0
    t0 = clock()

    def end_active(sid: int, status: str) -> None:
        nonlocal active_cells
        req = active.pop(sid)[0]
        active_cells -= float(req.dims[0]) * req.dims[1] * req.dims[2]
        batch.remove(sid)   # stream-ordered: behind the chunks and copies already queued
        req.status, req.done = status, clock() - t0

    def poll(wait_all: bool = False) -> None:
        keep = []
        for item in snaps:
            tk, req, step, buf, n, shape = item
            if batch.done(tk, wait=wait_all):
                if on_snapshot is not None:
                    on_snapshot(req, step, buf.view(shape).copy())
                req.snapshots.append(step)
                bufs.put(n, buf)
            else:
                keep.append(item)
        snaps[:] = keep
        keep = []
        for tk, req in finishing:
            if batch.done(tk, wait=wait_all):
                if req.status == "running":
                    req.status, req.done = "done", clock() - t0
            else:
                keep.append((tk, req))
        finishing[:] = keep

    try:
        while pending or queue or active or chunks or snaps or finishing:
            now = clock() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            # host-side cancellation and deadlines (queued or running)
            stop = control.take() if control is not None else set()
            for req in list(queue):
                if req.rid in stop or now > req.arrival + req.deadline:
                    queue.remove(req)
                    req.status, req.done = ("cancelled" if req.rid in stop else "deadline"), now
            for sid, (req, *_rest) in list(active.items()):
                if req.rid in stop or now > req.arrival + req.deadline:
                    end_active(sid, "cancelled" if req.rid in stop else "deadline")
            for req in list(r for r in pending if r.rid in stop):
                pending.remove(req)
                req.status, req.done = "cancelled", req.arrival
            # admit in policy order while the head fits the budget and the cap
            order_queue(queue, policy)
            admitted, limit = 0, (admit_per_turn if active else 1)
            while queue and admitted < limit:
                req = queue[0]
                need = batch.need_bytes(*req.dims)
                if need > budget_bytes:
                    queue.pop(0)  # can never fit
                    req.status = "rejected"
                    continue
                if batch.bytes + need > budget_bytes:
                    break
                cells = float(req.dims[0]) * req.dims[1] * req.dims[2]
                if max_active_cells is not None and active and active_cells + cells > max_active_cells:
                    break
                queue.pop(0)
                try:
                    if inputs is not None and req.rid in inputs:
                        p, codes, specs, src = inputs.pop(req.rid)
                    else:
                        p, codes, specs, src = build_inputs(req, Path(tmp.name) / str(req.rid))
                    sid = batch.add(p, codes, specs, req.steps, scheme=scheme)
                except (FdtdError, OSError, ValueError) as e:  # this request only
                    req.status, req.done, req.error = "failed", clock() - t0, str(e)
                    continue
                req.admitted = clock() - t0
                req.status = "running"
                active[sid] = [req, 0, src[2], p]
                active_cells += cells
                admitted += 1
            if active:
                # keep at most `inflight` chunks queued: wait for the oldest
                while len(chunks) >= inflight:
                    batch.done(chunks.popleft(), wait=True)
                batch.run(chunk)
                finished = []
                for sid, slot in active.items():
                    req, done, sz, _p = slot
                    adv = min(chunk, req.steps - done)
                    cell_updates += float(adv) * req.dims[0] * req.dims[1] * req.dims[2]
                    done += adv
                    slot[1] = done
                    if done % snapshot_every == 0 or done == req.steps:
                        ny, nx = req.dims[1], req.dims[0]
                        n = ny * nx
                        buf = bufs.get(n)
                        tk = batch.read_async(sid, "ez", buf.array, z0=sz, nplanes=1)
                        snaps.append((tk, req, done, buf, n, (ny, nx)))
                    if done >= req.steps:
                        finished.append(sid)
                chunks.append(batch.mark())
                for sid in finished:
                    req = active[sid][0]
                    if on_snapshot is not None and hasattr(on_snapshot, "final"):
                        on_snapshot.final(req, batch, sid)   # a synchronous read of the final state
                    finishing.append((batch.mark(), req))
                    req_cells = float(req.dims[0]) * req.dims[1] * req.dims[2]
                    active.pop(sid)
                    active_cells -= req_cells
                    batch.remove(sid)
            elif chunks:
                batch.done(chunks.popleft(), wait=True)
            elif pending and not queue and not snaps and not finishing:
                # idle until the next arrival
                time.sleep(max(0.0, min(0.05, pending[0].arrival - (clock() - t0))))
            poll(wait_all=not active and not pending and not queue)
        batch.synchronize()   # raises if a kernel gave up a bounded wait
        busy, span = batch.busy()
    finally:
        wall = clock() - t0
        batch.close()
        bufs.close()
        tmp.cleanup()
    return ServeResult(requests, wall, cell_updates, busy, span)
