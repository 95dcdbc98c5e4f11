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
