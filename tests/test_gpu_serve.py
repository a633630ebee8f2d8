"""Serving loop (lightning_gb300.serve): a Poisson request stream served with
continuous batching; every result must equal the same request computed
alone (forward values within 1e-12 x the Hamiltonian's coefficient norm,
against the per-gate API; adjoint values and Jacobians bit-identical to the
request run alone), and the timings must be causal."""
import numpy as np
import pytest

from helpers import assert_scalar
from lightning_gb300 import lightning_gb300_ops as ops
from lightning_gb300.serve import Server
from lightning_gb300.workloads import config4_packed

pytestmark = pytest.mark.gpu


def alone_forward(srv, r):
    p = srv.packed
    n = int(p.num_qubits[r])
    sv = ops.StateVectorC128(n)
    S = srv._ops_struct(r)
    for name, w, prm in zip(S.names, S.wires, S.params):
        getattr(sv, name)(w, False, prm)
    return float(ops.MeasurementsC128(sv).expval(srv._hamiltonian(r)))


def test_stream_results_equal_alone():
    packed, arrival, adjoint = config4_packed(rate=2000.0, duration=0.15, seed=11, n_max=16)
    srv = Server(128, adjoint_lanes=2)
    res = srv.run(packed, arrival, adjoint)
    R = packed.num_circuits
    assert R > 100 and np.all(np.isfinite(res.values))
    assert np.all(res.done >= res.start) and np.all(res.start >= res.arrival - 1e-6)
    s = res.summary()
    assert s["requests"] == R and s["p99_ms"] >= s["p50_ms"] > 0
    assert set(res.jacobians) == set(np.flatnonzero(adjoint).tolist())
    # forward requests: against the per-gate path, alone
    fwd = np.flatnonzero(~adjoint)
    for r in fwd[:: max(1, fwd.size // 12)]:
        ref = alone_forward(srv, int(r))
        norm = max(1.0, float(np.sum(np.abs(packed.term_coeffs[packed.term_offsets[r]:packed.term_offsets[r + 1]]))))
        assert_scalar(res.values[r], ref, np.complex128, mag=norm, what=f"request {r}")
    # forward requests batched differently give the same bits
    some = fwd[:20].tolist()
    again = srv.engines[0].run(packed.select(some))
    small = [k for k, r in enumerate(some) if packed.num_qubits[r] < srv.big]
    assert np.array_equal(again[small], res.values[np.array(some)[small]])
    # adjoint requests: alone equals in the mix
    adj = np.flatnonzero(adjoint)
    for r in adj[:: max(1, adj.size // 6)]:
        v, j = srv.adjoint_one(int(r))
        assert v == res.values[r] and np.array_equal(j, res.jacobians[int(r)])


def test_budget_limits_inflight():
    packed, arrival, adjoint = config4_packed(rate=4000.0, duration=0.05, seed=3, n_max=14)
    srv = Server(128, budget_bytes=4 * (1 << 14) * 16 * 3, adjoint_lanes=1)
    res = srv.run(packed, arrival, adjoint)
    assert np.all(np.isfinite(res.values))
    with pytest.raises(ValueError):
        srv.budget.acquire(srv.budget.total + 1)


def test_admission_control_under_overload():
    # a stream far beyond capacity with a 20 ms wait limit: requests are
    # refused once the lanes have measured rates; every admitted result is
    # the request's own, and refused requests have none
    packed, arrival, adjoint = config4_packed(rate=6000.0, duration=0.3, seed=21, n_max=20)
    srv = Server(128, adjoint_lanes=2, slo_s=0.02)
    res = srv.run(packed, arrival, adjoint)
    ok = res.admitted
    assert res.refused.any() and ok.sum() > 10
    assert np.all(np.isfinite(res.values[ok])) and np.all(np.isnan(res.values[~ok]))
    assert set(res.jacobians) == set(np.flatnonzero(adjoint & ok).tolist())
    s = res.summary()
    assert s["requests"] == int(ok.sum()) and s["refused"] == int((~ok).sum())
    fwd = np.flatnonzero(~adjoint & ok)
    for r in fwd[:: max(1, fwd.size // 6)]:
        ref = alone_forward(srv, int(r))
        norm = max(1.0, float(np.sum(np.abs(packed.term_coeffs[packed.term_offsets[r]:packed.term_offsets[r + 1]]))))
        assert_scalar(res.values[r], ref, np.complex128, mag=norm, what=f"request {r}")
