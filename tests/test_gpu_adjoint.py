"""GPU adjoint Jacobian vs the oracle, central finite differences and the
reference's known-answer values.

Known answers: pennylane_lightning/core/algorithms/tests/Test_AdjointJacobian.cpp
(:336-373 RX,RX,RX with Z@Z@Z; :375-431 mixed ops with X@X@X).
"""
import numpy as np
import pytest

from helpers import DTYPES, assert_close, obs_ns, rand_unitary, seed_of, sv_class

pytestmark = pytest.mark.gpu


def config0_ops(n, layers, rng):
    ops = []
    for _ in range(layers):
        for q in range(n):
            for g in ("RX", "RY", "RZ"):
                ops.append(dict(name=g, params=[float(rng.uniform(0, 2 * np.pi))], wires=[q]))
        for q in range(n):
            ops.append(dict(name="CNOT", wires=[q, (q + 1) % n]))
    return ops


def build_ops(ops_module, dt, ops):
    OS = ops_module.OpsStructC128 if np.dtype(dt) == np.complex128 else ops_module.OpsStructC64
    return OS([o["name"] for o in ops], [o.get("params", []) for o in ops], [o["wires"] for o in ops],
              [o.get("inverse", False) for o in ops], [o.get("matrix") for o in ops],
              [o.get("cwires", []) for o in ops], [o.get("cvals", []) for o in ops])


def gpu_jacobian(ops_module, dt, n, ops, obs_list, tp):
    sv = sv_class(ops_module, dt)(n)
    AJ = ops_module.AdjointJacobianC128 if np.dtype(dt) == np.complex128 else ops_module.AdjointJacobianC64
    jac = AJ()(sv, obs_list, build_ops(ops_module, dt, ops), tp, True)
    return np.asarray(jac, dtype=np.float64).reshape(len(obs_list), len(tp))


def sum_z(ops_module, dt, n):
    Named, _, Prod, Ham, _ = obs_ns(ops_module, dt)
    return Ham([1.0] * n, [Named("PauliZ", [q]) for q in range(n)])


def assert_jac(a, b, dt, what):
    # norm-relative over the Jacobian and relative per entry (entries below
    # the floor of the state check can be exact zeros)
    assert_close(np.asarray(a, np.float64), np.asarray(b, np.float64), dt, what=what)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", [4, 8, 12])
def test_config0_ansatz_vs_oracle(ops_module, oracle, dt, n):
    from oracle.pyoracle import pauli_sum_spec

    rng = np.random.default_rng(seed_of("adj0", n, dt.__name__))
    ops = config0_ops(n, 3, rng)
    npar = sum(1 for o in ops if o.get("params"))
    tp = list(range(npar))
    jg = gpu_jacobian(ops_module, dt, n, ops, [sum_z(ops_module, dt, n)], tp)
    jo = oracle.sv(n, dt).adjoint(ops, [pauli_sum_spec([(1.0, "Z", [q]) for q in range(n)])], tp, apply_ops=True)
    assert_jac(jg, jo, dt, "config0")


@pytest.mark.parametrize("dt", DTYPES)
def test_all_generators_multi_obs(ops_module, oracle, dt):
    from oracle.pyoracle import ObsData, pauli_sum_spec

    rng = np.random.default_rng(seed_of("adjgen", dt.__name__))
    n = 6
    ops = [dict(name="Hadamard", wires=[q]) for q in range(n)]
    for name, k in [("RX", 1), ("RY", 1), ("RZ", 1), ("PhaseShift", 1), ("IsingXX", 2), ("IsingXY", 2),
                    ("IsingYY", 2), ("IsingZZ", 2), ("CRX", 2), ("CRY", 2), ("CRZ", 2), ("ControlledPhaseShift", 2),
                    ("SingleExcitation", 2), ("SingleExcitationMinus", 2), ("SingleExcitationPlus", 2),
                    ("DoubleExcitation", 4), ("DoubleExcitationMinus", 4), ("DoubleExcitationPlus", 4),
                    ("PSWAP", 2), ("MultiRZ", 3), ("GlobalPhase", 1)]:
        w = [int(x) for x in rng.choice(n, size=k, replace=False)]
        ops.append(dict(name=name, params=[float(rng.uniform(0, 6.28))], wires=w, inverse=bool(rng.integers(0, 2))))
        ops.append(dict(name="CNOT", wires=[int(w[0]), int((w[0] + 1) % n)]))
    # controlled forms and a matrix op
    ops.append(dict(name="RY", params=[0.37], wires=[2], cwires=[0, 4], cvals=[True, False]))
    ops.append(dict(name="IsingXY", params=[0.41], wires=[1, 3], cwires=[5], cvals=[True]))
    ops.append(dict(name="QubitUnitary", wires=[0, 5], matrix=rand_unitary(rng, 2)))
    ops.append(dict(name="MultiRZ", params=[0.9], wires=[1, 2], cwires=[4], cvals=[True]))
    npar = sum(1 for o in ops if o.get("params"))
    tp = sorted(int(x) for x in rng.choice(npar, size=npar - 3, replace=False))
    Named, Herm, Prod, Ham, _ = obs_ns(ops_module, dt)
    H2 = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    H2 = H2 + H2.conj().T
    obs = [sum_z(ops_module, dt, n), Ham([0.3, -0.7], [Prod([Named("PauliX", [0]), Named("PauliY", [1])]),
                                                       Named("PauliZ", [3])]),
           Named("PauliX", [2]), Herm(H2, [1, 4])]
    od = ObsData()
    off = od.add_matrix(H2)
    specs = [pauli_sum_spec([(1.0, "Z", [q]) for q in range(n)]), pauli_sum_spec([(0.3, "XY", [0, 1]),
                                                                                  (-0.7, "Z", [3])]),
             "named PauliX 2", f"herm 2 1 4 {off}"]
    jg = gpu_jacobian(ops_module, dt, n, ops, obs, tp)
    jo = oracle.sv(n, dt).adjoint(ops, specs, tp, od=od, apply_ops=True)
    assert_jac(jg, jo, dt, "generators")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("with_two_bit_flips", [False, True])
def test_fused_register_sweep_generators(ops_module, oracle, dt, with_two_bit_flips):
    # One observable and Pauli-word generators only, on 11 qubits: the whole
    # reverse sweep runs as fused two-register tile passes with reductions in
    # register stages (flip on a register bit, Z-type without flip, controlled
    # generators with a projector).  IsingXX / IsingYY flip two bits: their
    # passes take the shared-memory two-register kernel, mixed with the
    # register passes in one sweep.
    from oracle.pyoracle import pauli_sum_spec

    rng = np.random.default_rng(seed_of("adjreg", dt.__name__, with_two_bit_flips))
    n = 11
    gates = [("RX", 1), ("RY", 1), ("RZ", 1), ("CRX", 2), ("CRY", 2), ("CRZ", 2), ("IsingZZ", 2), ("MultiRZ", 3)]
    if with_two_bit_flips:
        gates += [("IsingXX", 2), ("IsingYY", 2)]
    ops = [dict(name="Hadamard", wires=[q]) for q in range(n)]
    for _ in range(4):
        for name, k in gates:
            w = [int(x) for x in rng.choice(n, size=k, replace=False)]
            ops.append(dict(name=name, params=[float(rng.uniform(0, 6.28))], wires=w,
                            inverse=bool(rng.integers(0, 2))))
            ops.append(dict(name="CNOT", wires=[int(w[0]), int((w[0] + 3) % n)]))
        ops.append(dict(name="RY", params=[float(rng.uniform(0, 6.28))], wires=[int(rng.integers(0, n))],
                        cwires=[int(rng.integers(0, n))], cvals=[True]))
    # controlled-RY entries whose control equals the target are invalid: redraw
    for o in ops:
        if o.get("cwires") and o["cwires"][0] == o["wires"][0]:
            o["cwires"] = [(o["wires"][0] + 5) % n]
    npar = sum(1 for o in ops if o.get("params"))
    tp = list(range(npar))
    terms = [(float(rng.normal()), "".join(rng.choice(list("XYZ"), size=m)),
              [int(x) for x in rng.choice(n, size=m, replace=False)]) for m in (1, 2, 2, 3, 4)]
    Named, _, Prod, Ham, _ = obs_ns(ops_module, dt)
    H = Ham([t[0] for t in terms], [Prod([Named("Pauli" + c, [w]) for c, w in zip(t[1], t[2])]) for t in terms])
    jg = gpu_jacobian(ops_module, dt, n, ops, [H], tp)
    jo = oracle.sv(n, dt).adjoint(ops, [pauli_sum_spec(terms)], tp, apply_ops=True)
    assert_jac(jg, jo, dt, "fused register sweep")


def test_known_answers_rx_zzz(ops_module):
    # Test_AdjointJacobian.cpp:336-373 (values computed with parameter shift)
    Named, _, Prod, _, _ = obs_ns(ops_module, np.complex128)
    p = [-np.pi / 7, np.pi / 5, 2 * np.pi / 3]
    ops = [dict(name="RX", params=[p[i]], wires=[i]) for i in range(3)]
    obs = Prod([Named("PauliZ", [0]), Named("PauliZ", [1]), Named("PauliZ", [2])])
    j = gpu_jacobian(ops_module, np.complex128, 3, ops, [obs], [0, 1, 2])[0]
    np.testing.assert_allclose(j, [-0.1755096592645253, 0.26478810666384334, -0.6312451595102775], atol=1e-7)


def test_known_answers_mixed_xxx(ops_module):
    # Test_AdjointJacobian.cpp:375-431 (values from default.qubit adjoint)
    Named, _, Prod, _, _ = obs_ns(ops_module, np.complex128)
    p = [-np.pi / 7, np.pi / 5, 2 * np.pi / 3]
    cnot = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)
    ops = [dict(name="RZ", params=[p[0]], wires=[0]), dict(name="RY", params=[p[1]], wires=[0]),
           dict(name="RZ", params=[p[2]], wires=[0]), dict(name="QubitUnitary", wires=[0, 1], matrix=cnot),
           dict(name="CNOT", wires=[1, 2]), dict(name="RZ", params=[p[0]], wires=[1]),
           dict(name="RY", params=[p[1]], wires=[1]), dict(name="RZ", params=[p[2]], wires=[1])]
    obs = Prod([Named("PauliX", [0]), Named("PauliX", [1]), Named("PauliX", [2])])
    j = gpu_jacobian(ops_module, np.complex128, 3, ops, [obs], list(range(6)))[0]
    np.testing.assert_allclose(j, [0.0, -0.674214427, 0.275139672, 0.275139672, -0.0129093062, 0.323846156],
                               atol=1e-7)


def test_central_finite_differences(ops_module):
    # d<H>/dtheta_i = (<H>(theta + h e_i) - <H>(theta - h e_i)) / 2h, h = 1e-4
    rng = np.random.default_rng(seed_of("fd"))
    n = 6
    ops = config0_ops(n, 2, rng)
    idx = [i for i, o in enumerate(ops) if o.get("params")]
    tp = list(range(len(idx)))
    H = sum_z(ops_module, np.complex128, n)
    jac = gpu_jacobian(ops_module, np.complex128, n, ops, [H], tp)[0]

    def energy(ops_):
        sv = ops_module.StateVectorC128(n)
        for o in ops_:
            getattr(sv, o["name"])(o["wires"], False, o.get("params", []))
        return ops_module.MeasurementsC128(sv).expval(H)

    h = 1e-4
    for k in rng.choice(len(idx), size=8, replace=False):
        plus = [dict(o) for o in ops]
        minus = [dict(o) for o in ops]
        plus[idx[k]]["params"] = [ops[idx[k]]["params"][0] + h]
        minus[idx[k]]["params"] = [ops[idx[k]]["params"][0] - h]
        fd = (energy(plus) - energy(minus)) / (2 * h)
        assert abs(fd - jac[k]) < 1e-6, (k, fd, jac[k])
