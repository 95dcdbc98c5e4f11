"""Serving loop: continuous batching keeps each request's result identical to
running it alone, admits within the memory budget, streams snapshots."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from fdtd_gb300 import serve

pytestmark = pytest.mark.gpu


class Recorder:
    def __init__(self):
        self.planes = {}
        self.finals = {}

    def __call__(self, req, step, plane):
        self.planes[(req.rid, step)] = plane.copy()

    def final(self, req, batch, sid):
        self.finals[req.rid] = batch.fields(sid)


@pytest.mark.parametrize("kernel,policy", [(fg.KERNEL_SINGLE_PASS, "fifo"), (fg.KERNEL_COMPACT, "fifo"),
                                           (fg.KERNEL_COMPACT_R16, "fifo"),
                                           (fg.KERNEL_COMPACT, "sjf")])
def test_served_results_equal_lone_runs_and_overlap(cuda, tmp_path, kernel, policy):
    reqs = serve.poisson_stream(rate=40.0, duration=0.3, seed=3, dims=(24, 56), steps=(50, 150))
    assert len(reqs) >= 4
    for r in reqs:  # whole chunks keep the snapshot steps exact
        r.steps = (r.steps // 25) * 25 or 25
    rec = Recorder()
    budget = sum(fg.Batch.solve_bytes(*r.dims) for r in reqs[:3])  # forces queueing
    # sjf: also a cell cap that holds about two of these solves at a time
    cap = 2.0 * 40 ** 3 if policy == "sjf" else None
    res = serve.serve(reqs, budget_bytes=budget, chunk=25, snapshot_every=50, on_snapshot=rec, kernel=kernel,
                      policy=policy, max_active_cells=cap)
    s = res.summary()
    assert s["completed"] == len(reqs)
    # continuous batching: some request was admitted while another was still running
    spans = sorted((r.admitted, r.done) for r in reqs)
    assert any(spans[i + 1][0] < spans[i][1] for i in range(len(spans) - 1))
    for r in reqs:
        assert r.snapshots[-1] == r.steps
        p, codes, specs, src = serve.build_inputs(r, tmp_path / f"alone{r.rid}")
        with fg.Solver(p, codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel) as alone:
            alone.run(r.steps)
            want = alone.fields()
        got = rec.finals[r.rid]
        for name in want:
            assert np.array_equal(got[name].view(np.uint32), want[name].view(np.uint32)), (r.rid, name)
        assert np.array_equal(rec.planes[(r.rid, r.steps)], want["ez"][src[2]])
    assert s["p50_ms"] > 0 and s["p99_ms"] >= s["p50_ms"]


class Canceller(Recorder):
    """Cancels request `victim` from the host when its first snapshot arrives."""

    def __init__(self, control, victim):
        super().__init__()
        self.control, self.victim = control, victim

    def __call__(self, req, step, plane):
        super().__call__(req, step, plane)
        if req.rid == self.victim:
            self.control.cancel(req.rid)


def test_cancel_mid_run_and_deadline_leave_other_requests_unaffected(cuda, tmp_path):
    reqs = serve.poisson_stream(rate=40.0, duration=0.3, seed=5, dims=(24, 48), steps=(100, 200))
    assert len(reqs) >= 4
    for r in reqs:
        r.steps = (r.steps // 25) * 25
    victim = reqs[0].rid
    reqs[0].steps = 1000          # long enough to be cancelled while it runs
    reqs[1].deadline = 0.0        # ends at once (queued or running)
    ctl = serve.ServeControl()
    rec = Canceller(ctl, victim)
    res = serve.serve(reqs, budget_bytes=10 ** 10, chunk=25, snapshot_every=50, on_snapshot=rec,
                      kernel=fg.KERNEL_COMPACT, control=ctl)
    s = res.summary()
    assert reqs[0].status == "cancelled" and reqs[0].snapshots and reqs[0].snapshots[-1] < 1000
    assert reqs[1].status == "deadline"
    assert s["cancelled"] == 1 and s["deadline"] == 1 and s["completed"] == len(reqs) - 2
    assert 0.0 < s["gpu_busy_fraction"] <= 1.0 + 1e-6
    for r in reqs[2:]:
        assert r.status == "done" and r.snapshots[-1] == r.steps
        p, codes, specs, src = serve.build_inputs(r, tmp_path / f"alone{r.rid}")
        with fg.Solver(p, codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=fg.KERNEL_COMPACT) as alone:
            alone.run(r.steps)
            want = alone.fields()
        got = rec.finals[r.rid]
        for name in want:
            assert np.array_equal(got[name].view(np.uint32), want[name].view(np.uint32)), (r.rid, name)


def test_batch_async_reads_and_tickets(cuda, tmp_path):
    """fdtd_batch_read_async returns the planes as they are after the steps
    queued before it, while later steps are already queued behind it."""
    reqs = serve.poisson_stream(rate=40.0, duration=0.2, seed=9, dims=(24, 40), steps=(100, 100))[:2]
    b = fg.Batch(0, fg.KERNEL_COMPACT_R16)
    ids, inp = [], []
    for r in reqs:
        p, codes, specs, src = serve.build_inputs(r, tmp_path / str(r.rid))
        ids.append(b.add(p, codes, specs, 60, scheme=fg.SCHEME_CORRECTED))
        inp.append((p, codes, specs, src))
    b.run(30)
    bufs = [fg.PinnedBuffer(r.dims[0] * r.dims[1]) for r in reqs]
    tks = [b.read_async(sid, "ez", buf.array, z0=src[2], nplanes=1) for sid, buf, (_, _, _, src)
           in zip(ids, bufs, inp)]
    b.run(30)
    end = b.mark()
    assert b.done(end, wait=True)
    for tk, buf, r, (p, codes, specs, src) in zip(tks, bufs, reqs, inp):
        assert b.done(tk)
        with fg.Solver(p, codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=fg.KERNEL_COMPACT_R16) as alone:
            alone.run(30)
            want = alone.field("ez")[src[2]]
        got = buf.view((r.dims[1], r.dims[0]))
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert b.steps(ids[0]) == 60
    b.close()
    for buf in bufs:
        buf.close()
