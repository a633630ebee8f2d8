"""Host-side pieces of the request server (no GPU needed): the device-memory
budget that admits requests, and the latency / throughput summary that the
serving measurement reports."""
import threading
import time

import numpy as np
import pytest

from lightning_gb300.serve import MemoryBudget, ServeResult


def test_budget_admits_within_total_and_rejects_oversized():
    b = MemoryBudget(100)
    assert b.acquire(60, block=False)
    assert not b.acquire(50, block=False)  # 40 left
    assert b.acquire(40, block=False)
    assert b.free == 0
    b.release(60)
    assert b.acquire(50, block=False) and b.free == 10
    with pytest.raises(ValueError):
        b.acquire(101)  # can never fit: an error, not a wait


def test_blocking_acquire_waits_for_a_release():
    b = MemoryBudget(10)
    assert b.acquire(10)
    got = threading.Event()

    def waiter():
        b.acquire(6)
        got.set()

    t = threading.Thread(target=waiter, daemon=True)
    t.start()
    time.sleep(0.05)
    assert not got.is_set()  # still waiting: nothing released yet
    b.release(5)
    time.sleep(0.05)
    assert not got.is_set()  # 5 free, 6 wanted
    b.release(5)
    assert got.wait(2.0)
    t.join(2.0)
    assert b.free == 4


def test_summary_latency_and_throughput():
    arrival = np.array([0.0, 0.1, 0.2, 0.3])
    done = np.array([0.5, 0.6, 1.0, 2.3])
    r = ServeResult(values=np.zeros(4), jacobians={}, arrival=arrival, start=arrival.copy(), done=done,
                    lane=np.zeros(4, np.int32), batches=[(0, 2, 0.4), (1, 2, 1.0)])
    s = r.summary()
    lat = done - arrival
    assert s["requests"] == 4
    assert s["p50_ms"] == pytest.approx(np.percentile(lat, 50) * 1e3)
    assert s["p99_ms"] == pytest.approx(np.percentile(lat, 99) * 1e3)
    assert s["span_s"] == pytest.approx(2.3)
    assert s["throughput_per_s"] == pytest.approx(4 / 2.3)
    assert s["mean_batch"] == pytest.approx(2.0) and s["batches"] == 2
