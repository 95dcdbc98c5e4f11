"""Admission order of the serving loop (host logic, no GPU)."""
from __future__ import annotations

import pytest

from fdtd_gb300 import serve


def _req(rid, arrival, dims, steps):
    return serve.Request(rid, arrival, dims, 1.0e9, steps, 0)


def test_fifo_keeps_arrival_order_and_sjf_puts_least_work_first():
    q = [_req(0, 0.1, (64, 64, 64), 1000), _req(1, 0.2, (32, 32, 32), 4000), _req(2, 0.3, (128, 64, 64), 500),
         _req(3, 0.4, (32, 32, 32), 4000)]
    fifo = list(q)
    serve.order_queue(fifo, "fifo")
    assert [r.rid for r in fifo] == [0, 1, 2, 3]
    sjf = list(q)
    serve.order_queue(sjf, "sjf")
    # work: 0 -> 2.6e8, 1 -> 1.3e8, 2 -> 2.6e8, 3 -> 1.3e8; ties by arrival
    assert [r.rid for r in sjf] == [1, 3, 0, 2]
    assert serve.work(q[2]) == 128 * 64 * 64 * 500
    with pytest.raises(ValueError):
        serve.order_queue(list(q), "lifo")
