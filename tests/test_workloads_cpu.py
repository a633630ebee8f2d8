"""The seeded synthetic workloads have the shapes of the benchmark
configurations (no GPU needed): gate counts, parameter counts, observable
sizes, the config-1 CZ pairing across the high index bits, the config-4
request mix, and the per-step algorithmic bytes the headline metric uses."""
import numpy as np
import pytest

from lightning_gb300.workloads import config0, config1, config3, config4_packed, unfused_bytes


def test_config0_hardware_efficient_ansatz():
    ops = config0(20, 10, seed=1000)
    rot = [o for o in ops if o.name in ("RX", "RY", "RZ")]
    cnot = [o for o in ops if o.name == "CNOT"]
    assert len(rot) == 600 and len(cnot) == 200 and len(ops) == 800
    assert all(0.0 <= o.params[0] < 2 * np.pi for o in rot)
    assert {tuple(o.wires) for o in cnot[:20]} == {(q, (q + 1) % 20) for q in range(20)}


def test_config1_random_circuit_shape_and_bytes():
    ops, ham = config1(30, 20, seed=1001)
    su2 = [o for o in ops if o.name == "QubitUnitary"]
    cz = [o for o in ops if o.name == "CZ"]
    assert len(su2) == 600 and len(cz) == 300
    for o in su2[:50]:
        m = o.matrix
        assert np.allclose(m @ m.conj().T, np.eye(2), atol=1e-12)
        assert abs(np.linalg.det(m) - 1.0) < 1e-12  # SU(2)
    for c in range(20):
        pairs = [tuple(o.wires) for o in cz[15 * c:15 * (c + 1)]]
        wires = [w for p in pairs for w in p]
        assert sorted(wires) == list(range(30))  # disjoint pairs over all wires
        for a, b in pairs:
            assert not (a >= 24 and b >= 24)  # every wire >= 24 meets one below
    assert len(ham.coeffs) == 64
    assert all(1 <= len(w) <= 4 and len(set(w)) == len(w) for w in ham.wires)
    # the headline metric's bytes per step: 2 N S per dense gate, 1/4 of it per CZ
    assert unfused_bytes(ops, 30, 16) == pytest.approx(23192823398400.0)


def test_config3_parameters_and_entanglers():
    ops, ham = config3(28, 12, seed=1003)
    rot = [o for o in ops if o.name in ("RZ", "RY")]
    cnot = [o for o in ops if o.name == "CNOT"]
    assert len(rot) == 1008 and len(cnot) == 336
    for layer in range(12):
        r = layer % 27 + 1
        assert {tuple(o.wires) for o in cnot[28 * layer:28 * (layer + 1)]} == {(q, (q + r) % 28) for q in range(28)}
    assert len(ham.coeffs) == 200 and all(1 <= len(w) <= 4 for w in ham.wires)


def test_config4_request_stream():
    packed, arrival, adjoint = config4_packed(duration=2.0)
    R = packed.num_circuits
    assert R == arrival.size == adjoint.size
    assert abs(R - 4000) < 4 * np.sqrt(4000)  # Poisson at 2000 requests/s for 2 s
    assert np.all(np.diff(arrival) >= 0) and 0 <= arrival[0] and arrival[-1] < 2.0
    ns = np.asarray(packed.num_qubits)
    assert ns.min() >= 8 and ns.max() <= 26
    assert np.mean(ns <= 12) > np.mean(ns >= 22)  # P(n) ~ 2^(-n/4): small registers dominate
    assert abs(adjoint.mean() - 0.3) < 0.03
    nops = np.diff(np.asarray(packed.op_offsets))
    depth = nops / (4 * ns)
    assert np.all(depth == np.round(depth)) and depth.min() >= 2 and depth.max() <= 12
