"""VectorJacobianProductC* (LQubitBindings.hpp:412-457): w_j = <dy | d psi /
d theta_j>.  Checked two ways: with dy = H psi, 2 Re w equals the adjoint
Jacobian of <H> (tolerance 1e-12 / 1e-5 relative); with a random dy, w
equals central finite differences of the state (h = 1e-4, 1e-7 absolute)."""
import numpy as np
import pytest

from helpers import assert_close, seed_of

pytestmark = pytest.mark.gpu

CIRCUIT = [("RX", [0], 0.3), ("RY", [1], -1.1), ("CNOT", [0, 1], None), ("IsingXY", [1, 2], 0.7),
           ("RZ", [2], 2.2), ("PhaseShift", [0], 0.4), ("CRY", [2, 0], -0.6), ("SingleExcitation", [0, 2], 1.3),
           ("Hadamard", [1], None), ("MultiRZ", [0, 1, 2], 0.9), ("RY", [2], 0.25)]


def build(ops_module, prec, thetas, n=3):
    OS = ops_module.OpsStructC128 if prec == 128 else ops_module.OpsStructC64
    SV = ops_module.StateVectorC128 if prec == 128 else ops_module.StateVectorC64
    names, params, wires, k = [], [], [], 0
    for name, w, p in CIRCUIT:
        names.append(name)
        wires.append(w)
        if p is None:
            params.append([])
        else:
            params.append([float(thetas[k])])
            k += 1
    S = OS(names, params, wires, [False] * len(names), [None] * len(names))
    sv = SV(n)
    for name, w, p in zip(names, wires, params):
        sv.applyOperation(name, w, False, p)
    return sv, S


def thetas0():
    return np.array([p for _, _, p in CIRCUIT if p is not None])


@pytest.mark.parametrize("prec,tol", [(128, 1e-12), (64, 1e-5)])
def test_vjp_with_h_psi_matches_adjoint(ops_module, prec, tol):
    th = thetas0()
    sv, S = build(ops_module, prec, th)
    s = "C128" if prec == 128 else "C64"
    NO, TP, HA = (getattr(ops_module.observables, k + s) for k in ("NamedObs", "TensorProdObs", "Hamiltonian"))
    H = HA([0.5, -1.2, 0.8], [TP([NO("PauliZ", [0]), NO("PauliX", [2])]), NO("PauliY", [1]),
                              TP([NO("PauliX", [0]), NO("PauliZ", [1])])])
    psi = sv.state()
    dt = psi.dtype
    # H psi on the host
    I, X, Y, Z = (np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.diag([1.0, -1.0]))
    def kron(*m):
        out = np.eye(1)
        for a in m:
            out = np.kron(out, a)
        return out
    Hm = 0.5 * kron(Z, I, X) - 1.2 * kron(I, Y, I) + 0.8 * kron(X, Z, I)
    dy = (Hm @ psi.astype(np.complex128)).astype(dt)
    tp = list(range(th.size))
    w = getattr(ops_module.algorithms, "VectorJacobianProduct" + s)()(sv, S, dy, tp)
    jac = getattr(ops_module.algorithms, "AdjointJacobian" + s)()(sv, [H], S, tp)
    assert_close(2 * w.real, np.asarray(jac).ravel(), dt, what="2 Re VJP vs Jacobian")


def test_vjp_matches_finite_differences(ops_module):
    rng = np.random.default_rng(seed_of("vjp-fd"))
    th = thetas0()
    sv, S = build(ops_module, 128, th)
    dy = rng.normal(size=8) + 1j * rng.normal(size=8)
    w = ops_module.algorithms.VectorJacobianProductC128()(sv, S, dy, list(range(th.size)))
    h = 1e-4
    for j in range(th.size):
        tp, tm = th.copy(), th.copy()
        tp[j] += h
        tm[j] -= h
        dpsi = (build(ops_module, 128, tp)[0].state() - build(ops_module, 128, tm)[0].state()) / (2 * h)
        assert abs(np.vdot(dy, dpsi) - w[j]) < 1e-7, j


def test_vjp_subset_and_errors(ops_module):
    th = thetas0()
    sv, S = build(ops_module, 128, th)
    dy = np.ones(8, np.complex128)
    full = ops_module.algorithms.VectorJacobianProductC128()(sv, S, dy, list(range(th.size)))
    part = ops_module.algorithms.VectorJacobianProductC128()(sv, S, dy, [1, 4])
    assert np.allclose(part, full[[1, 4]], atol=1e-14)
    assert ops_module.algorithms.VectorJacobianProductC128()(sv, S, dy, []).shape == (0,)
    with pytest.raises(ops_module.LightningException):
        ops_module.algorithms.VectorJacobianProductC128()(sv, S, np.ones(4), [0])


def _oracle_circuit(rng, n):
    # plain, two-wire, multi-wire and controlled generators, some inverted
    ops = []
    for layer in range(3):
        for q in range(n):
            ops.append(dict(name=str(rng.choice(["RX", "RY", "RZ", "PhaseShift"])), wires=[q],
                            params=[float(rng.uniform(0, 2 * np.pi))], inverse=bool(rng.integers(0, 2))))
        ops.append(dict(name="CNOT", wires=[layer % n, (layer + 1) % n], params=[]))
        ops.append(dict(name="IsingXX", wires=[0, n - 1], params=[float(rng.uniform(0, 6))]))
        ops.append(dict(name="CRY", wires=[1, 2], params=[float(rng.uniform(0, 6))], inverse=True))
        ops.append(dict(name="MultiRZ", wires=[0, 2, 3], params=[float(rng.uniform(0, 6))]))
        ops.append(dict(name="RX", wires=[3], params=[float(rng.uniform(0, 6))], cwires=[0, 4], cvals=[True, False]))
    return ops


@pytest.mark.parametrize("prec,tol", [(128, 1e-12), (64, 1e-5)])
def test_vjp_matches_oracle(ops_module, oracle, prec, tol):
    # against the oracle's restatement of VectorJacobianProduct.hpp:79-160,
    # itself pinned to the reference's build
    from helpers import rand_state

    rng = np.random.default_rng(seed_of("vjp-oracle", prec))
    n = 5
    ops = _oracle_circuit(rng, n)
    dt = np.complex128 if prec == 128 else np.complex64
    s = "C128" if prec == 128 else "C64"
    OS = getattr(ops_module, "OpsStruct" + s)
    S = OS([o["name"] for o in ops], [o["params"] for o in ops], [o["wires"] for o in ops],
           [o.get("inverse", False) for o in ops], [None] * len(ops), [o.get("cwires", []) for o in ops],
           [o.get("cvals", []) for o in ops])
    sv = getattr(ops_module, "StateVector" + s)(n)
    for o in ops:
        sv.applyOperation(o["name"], o["wires"], o.get("inverse", False), o["params"], o.get("cwires", ()),
                          o.get("cvals", ()))
    npar = sum(1 for o in ops if o["params"])
    tp = sorted(int(x) for x in rng.choice(npar, size=npar // 2, replace=False))
    dy = rand_state(rng, n, dt)
    w = getattr(ops_module.algorithms, "VectorJacobianProduct" + s)()(sv, S, dy, tp)
    ref = oracle.sv(n, dt).vjp(ops, dy.astype(np.complex128), tp, apply_ops=True)
    assert np.asarray(w).shape == (len(tp),)
    assert_close(np.asarray(w), ref, dt, what="VJP vs oracle")
