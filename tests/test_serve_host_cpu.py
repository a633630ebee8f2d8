"""Host-side pieces of the request server (no GPU needed): the device-memory
budget that admits requests, and the latency / throughput summary that the
serving measurement reports."""
import threading
import time

import numpy as np
import pytest

from lightning_gb300.serve import Admission, MemoryBudget, ServeResult


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


def test_summary_excludes_refused_requests():
    arrival = np.array([0.0, 0.1, 0.2, 0.3])
    done = np.array([0.5, 0.1, 1.0, 0.3])
    refused = np.array([False, True, False, True])
    r = ServeResult(values=np.zeros(4), jacobians={}, arrival=arrival, start=arrival.copy(), done=done,
                    lane=np.zeros(4, np.int32), batches=[(0, 1, 0.5), (2, 1, 0.8)], refused=refused)
    s = r.summary()
    assert s["requests"] == 2 and s["offered"] == 4 and s["refused"] == 2
    assert s["p50_ms"] == pytest.approx(np.percentile([0.5, 0.8], 50) * 1e3)
    assert s["span_s"] == pytest.approx(1.0) and s["throughput_per_s"] == pytest.approx(2.0)
    assert s["lanes"]["forward"]["lane_seconds"] == pytest.approx(0.5)
    assert s["lanes"]["adjoint"]["requests"] == 1


def test_admission_admits_until_a_rate_is_known():
    a = Admission(0.5, [1, 1, 4])
    assert all(a.offer(0, 1e9) for _ in range(10))  # no completed batch yet: no estimate
    assert a.backlog[0] == pytest.approx(1e10)


def test_admission_refuses_beyond_the_predicted_wait():
    a = Admission(1.0, [1, 1, 4])
    assert a.offer(0, 100.0)
    a.completed(0, 100.0, 1.0)  # 100 units/s on the one lane of kind 0
    assert a.rate[0] == pytest.approx(100.0) and a.backlog[0] == pytest.approx(0.0)
    assert a.offer(0, 60.0)  # 0.6 s of work ahead of nothing
    assert not a.offer(0, 60.0)  # 1.2 s > 1 s: refused, backlog unchanged
    assert a.backlog[0] == pytest.approx(60.0)
    assert a.offer(0, 30.0)  # 0.9 s
    # kind 2 has 4 lanes: a batch of 100 units in 1 s is 400 units/s for the kind
    assert a.offer(2, 100.0)
    a.completed(2, 100.0, 1.0)
    assert a.rate[2] == pytest.approx(400.0)
    assert a.offer(2, 350.0) and not a.offer(2, 100.0)
    # the rate follows new batches with weight 0.2
    a.completed(0, 90.0, 0.3)  # 300 units/s
    assert a.rate[0] == pytest.approx(0.8 * 100.0 + 0.2 * 300.0)


def test_admission_without_slo_admits_everything():
    a = Admission(None, [1])
    a.offer(0, 1.0)
    a.completed(0, 1.0, 10.0)
    assert all(a.offer(0, 1e12) for _ in range(5))
