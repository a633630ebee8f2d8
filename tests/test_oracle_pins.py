"""CPU tests that pin the oracle (the LM restatement in oracle/lm_oracle.hpp).

1. Against the golden fixtures generated from the reference's own C++
   (tests/golden/make_golden.py) — runs everywhere.
2. Against the reference shim directly, on fresh random inputs — runs where
   oracle/_ref/libplref.so could be built from the reference checkout.
3. Against the reference's own known-answer values
   (core/algorithms/tests/Test_AdjointJacobian.cpp:336-431).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from gate_table import CONTROLLED_GATES, CONTROLLED_GENERATORS, GATES, GENERATORS, gate_params, gate_wires
from helpers import assert_close, assert_scalar, rand_state, rand_unitary, seed_of

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_lq.npz"
DT = {"c128": np.complex128, "c64": np.complex64}


@pytest.fixture(scope="module")
def golden():
    g = np.load(GOLDEN)
    return g, json.loads(str(g["meta"]))


def _ref():
    from oracle.pyoracle import Oracle, available

    if not available("ref"):
        pytest.skip("reference shim not built here (no reference checkout)")
    return Oracle("ref")


@pytest.mark.parametrize("tag", ["c128", "c64"])
def test_golden_gates(oracle, golden, tag):
    g, meta = golden
    dt = DT[tag]
    st = g[f"state_in_{tag}"]
    n = 5
    checked = 0
    for key, m in meta.items():
        if not key.startswith((f"gate_{tag}_", f"cgate_{tag}_", f"gen_{tag}_", f"cgen_{tag}_", f"mat_{tag}_")):
            continue
        o = oracle.sv(n, dt)
        o.set_state(st)
        kind = key.split("_")[0]
        if kind == "gate":
            o.apply(key.split("_")[2], m["wires"], m["inverse"], m["params"])
        elif kind == "cgate":
            o.apply(key.split("_")[2], m["wires"], False, m["params"], m["cwires"], m["cvals"])
        elif kind == "gen":
            assert o.apply_generator(key.split("_")[2], m["wires"]) == m["scale"]
        elif kind == "cgen":
            assert o.apply_generator(key.split("_")[2], m["wires"], False, m["cwires"], m["cvals"]) == m["scale"]
        else:
            o.apply_matrix(g[key + "_U"], m["wires"], m["inverse"])
        assert_close(o.state(), g[key], dt, what=key)
        checked += 1
    assert checked > 130


@pytest.mark.parametrize("tag", ["c128", "c64"])
def test_golden_measurements(oracle, golden, tag):
    g, meta = golden
    dt = DT[tag]
    o = oracle.sv(5, dt)
    o.set_state(g[f"state_in_{tag}"])
    for i in range(8):
        assert_close(o.probs(meta[f"probs_{tag}_{i}"]["wires"]), g[f"probs_{tag}_{i}"], dt, what=f"probs {i}")
    for name in ("PauliX", "PauliY", "PauliZ", "Hadamard"):
        for w in range(5):  # one-wire observables have norm 1
            assert_scalar(o.expval_named(name, [w]), g[f"expval_{tag}_{name}"][w], dt, mag=1.0, what=f"E {name}{w}")
    from oracle.pyoracle import pauli_sum_spec

    spec = pauli_sum_spec([tuple(t) for t in meta[f"ham_{tag}"]["terms"]])
    c1 = sum(abs(t[0]) for t in meta[f"ham_{tag}"]["terms"])  # error scale of a Pauli-sum expectation
    assert_scalar(o.expval_obs(spec), g[f"ham_{tag}"][0], dt, mag=c1, what="E ham")
    assert_scalar(o.var_obs(spec), g[f"ham_{tag}"][1], dt, mag=c1 * c1, what="V ham")
    # seeded samples: exact integers
    assert np.array_equal(o.samples(2000, 37), g[f"samples_{tag}"])
    assert np.array_equal(o.samples(2000, 37, [3, 0]), g[f"samples_w_{tag}"])
    # Metropolis-Hastings (MeasurementsLQubit.hpp:551-594): exact integers
    for kname in ("Local", "NonZeroRandom"):
        assert np.array_equal(o.mcmc_samples(kname, 50, 1500, 91), g[f"mcmc_{kname}_{tag}"]), kname


def test_golden_config0_small(oracle, golden):
    from lightning_gb300.workloads import config0, sum_z
    from oracle.pyoracle import pauli_sum_spec

    g, _ = golden
    circuit = config0(8, 3, seed=1000)
    o = oracle.sv(8, np.complex128)
    for op in circuit:
        o.apply(op.name, op.wires, False, op.params)
    st = o.state()
    assert_close(st[g["config0_small_idx"]], g["config0_small_amps"], np.complex128, what="state")
    spec = pauli_sum_spec(sum_z(8).terms())
    assert_scalar(o.expval_obs(spec), g["config0_small_expval"][0], np.complex128, mag=8.0)  # sum |c| = 8
    tp = list(range(sum(1 for op in circuit if op.params)))
    jac = oracle.sv(8, np.complex128).adjoint([op.as_dict() for op in circuit], [spec], tp, apply_ops=True)[0]
    assert_close(jac, g["config0_small_jac"], np.complex128, what="config-0 Jacobian")


def test_golden_config1_config3_small(oracle, golden):
    from lightning_gb300.workloads import config1, config3
    from oracle.pyoracle import pauli_sum_spec

    g, _ = golden
    circuit, ham = config1(12, 4, seed=1001)
    o = oracle.sv(12, np.complex128)
    for op in circuit:
        if op.matrix is not None:
            o.apply_matrix(op.matrix, op.wires, False)
        else:
            o.apply(op.name, op.wires, False, op.params)
    assert_close(o.state(), g["config1_small_state"], np.complex128, what="config1 state")
    assert_scalar(o.expval_obs(pauli_sum_spec(ham.terms())), g["config1_small_expval"][0], np.complex128,
                  mag=float(np.sum(np.abs(ham.coeffs))))
    circuit, ham = config3(8, 3, seed=1003, nterms=20)
    tp = list(range(sum(1 for op in circuit if op.params)))
    jac = oracle.sv(8, np.complex128).adjoint([op.as_dict() for op in circuit], [pauli_sum_spec(ham.terms())], tp,
                                              apply_ops=True)[0]
    assert_close(jac, g["config3_small_jac"], np.complex128, what="config-3 Jacobian")


def test_known_answers_adjoint(oracle):
    # Test_AdjointJacobian.cpp:336-373 and :375-431
    p = [-np.pi / 7, np.pi / 5, 2 * np.pi / 3]
    ops = [dict(name="RX", params=[p[i]], wires=[i]) for i in range(3)]
    j = oracle.sv(3).adjoint(ops, ["prod 3 named PauliZ 0 named PauliZ 1 named PauliZ 2"], [0, 1, 2], apply_ops=True)
    np.testing.assert_allclose(j[0], [-0.1755096592645253, 0.26478810666384334, -0.6312451595102775], atol=1e-7)
    cnot = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)
    ops = [dict(name="RZ", params=[p[0]], wires=[0]), dict(name="RY", params=[p[1]], wires=[0]),
           dict(name="RZ", params=[p[2]], wires=[0]), dict(name="QubitUnitary", wires=[0, 1], matrix=cnot),
           dict(name="CNOT", wires=[1, 2]), dict(name="RZ", params=[p[0]], wires=[1]),
           dict(name="RY", params=[p[1]], wires=[1]), dict(name="RZ", params=[p[2]], wires=[1])]
    j = oracle.sv(3).adjoint(ops, ["prod 3 named PauliX 0 named PauliX 1 named PauliX 2"], list(range(6)),
                             apply_ops=True)
    np.testing.assert_allclose(j[0], [0.0, -0.674214427, 0.275139672, 0.275139672, -0.0129093062, 0.323846156],
                               atol=1e-7)


# ---------------------------------------------------------------- direct pins vs the reference shim
@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
def test_restatement_vs_reference_gates(oracle, dt):
    ref = _ref()
    rng = np.random.default_rng(seed_of("pin-gates", dt.__name__))
    n = 6
    for name in GATES:
        for inv in (False, True):
            st = rand_state(rng, n, dt)
            w = gate_wires(name, rng, n)
            p = gate_params(name, rng)
            a, b = oracle.sv(n, dt), ref.sv(n, dt)
            a.set_state(st)
            b.set_state(st)
            a.apply(name, w, inv, p)
            b.apply(name, w, inv, p)
            assert_close(a.state(), b.state(), dt, what=name)
    for name in CONTROLLED_GATES:
        nwk = GATES[name][0] or 2
        ws = [int(x) for x in rng.choice(n, size=nwk + 2, replace=False)]
        cv = [bool(x) for x in rng.integers(0, 2, size=2)]
        p = gate_params(name, rng)
        st = rand_state(rng, n, dt)
        a, b = oracle.sv(n, dt), ref.sv(n, dt)
        a.set_state(st)
        b.set_state(st)
        a.apply(name, ws[:nwk], True, p, ws[nwk:], cv)
        b.apply(name, ws[:nwk], True, p, ws[nwk:], cv)
        assert_close(a.state(), b.state(), dt, what="C" + name)
    for name in GENERATORS:
        w = gate_wires(name, rng, n)
        st = rand_state(rng, n, dt)
        a, b = oracle.sv(n, dt), ref.sv(n, dt)
        a.set_state(st)
        b.set_state(st)
        assert a.apply_generator(name, w) == b.apply_generator(name, w)
        assert_close(a.state(), b.state(), dt, what="gen " + name)
    for name in CONTROLLED_GENERATORS:
        nwk = GATES[name][0] or 2
        ws = [int(x) for x in rng.choice(n, size=nwk + 1, replace=False)]
        st = rand_state(rng, n, dt)
        a, b = oracle.sv(n, dt), ref.sv(n, dt)
        a.set_state(st)
        b.set_state(st)
        assert a.apply_generator(name, ws[:nwk], False, ws[nwk:], [True]) == \
            b.apply_generator(name, ws[:nwk], False, ws[nwk:], [True])
        assert_close(a.state(), b.state(), dt, what="cgen " + name)


@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
def test_restatement_vs_reference_measurements(oracle, dt):
    from oracle.pyoracle import ObsData, pauli_sum_spec

    ref = _ref()
    rng = np.random.default_rng(seed_of("pin-meas", dt.__name__))
    n = 7
    st = rand_state(rng, n, dt)
    a, b = oracle.sv(n, dt), ref.sv(n, dt)
    a.set_state(st)
    b.set_state(st)
    for wires in (None, [3], [6, 1], [2, 5, 0], list(range(n))[::-1]):
        assert_close(a.probs(wires), b.probs(wires), dt)
    for k in (1, 2, 3, 4):
        U = rand_unitary(rng, k)
        H = U + U.conj().T
        w = [int(x) for x in rng.choice(n, size=k, replace=False)]
        assert_scalar(a.expval_matrix(H, w), b.expval_matrix(H, w), dt, mag=float(np.linalg.norm(H, 2)))
    terms = [(float(rng.normal()), "".join(rng.choice(list("XYZ"), size=m)),
              [int(x) for x in rng.choice(n, size=m, replace=False)]) for m in (1, 2, 3, 4)]
    spec = pauli_sum_spec(terms)
    c1 = sum(abs(t[0]) for t in terms)
    assert_scalar(a.expval_obs(spec), b.expval_obs(spec), dt, mag=c1)
    od = ObsData()
    H1 = rand_unitary(rng, 1) + rand_unitary(rng, 1).conj().T
    off = od.add_matrix(H1)
    spec2 = f"ham 2 0.5 prod 2 named PauliX 0 herm 1 3 {off} -1.25 named Hadamard 2"
    c2 = 0.5 * float(np.linalg.norm(H1, 2)) + 1.25  # sum of |c| x term norms; var error scales with its square
    assert_scalar(a.var_obs(spec2, od), b.var_obs(spec2, od), dt, mag=c2 * c2)
    assert np.array_equal(a.samples(3000, 11), b.samples(3000, 11))
    # MCMC on a state with zeros (the non-zero-random kernel skips them)
    st0 = st.copy()
    st0[rng.random(st0.size) < 0.4] = 0
    st0 = (st0 / np.linalg.norm(st0)).astype(dt)
    a.set_state(st0)
    b.set_state(st0)
    for kname in ("Local", "NonZeroRandom", "other"):
        for burnin, shots in ((0, 700), (33, 500)):
            assert np.array_equal(a.mcmc_samples(kname, burnin, shots, 5), b.mcmc_samples(kname, burnin, shots, 5))


def test_restatement_vs_reference_adjoint(oracle):
    from lightning_gb300.workloads import config3
    from oracle.pyoracle import pauli_sum_spec

    ref = _ref()
    circuit, ham = config3(6, 2, seed=5, nterms=15)
    tp = list(range(0, sum(1 for op in circuit if op.params), 2))
    ops = [op.as_dict() for op in circuit]
    specs = [pauli_sum_spec(ham.terms()), "named PauliX 1"]
    ja = oracle.sv(6).adjoint(ops, specs, tp, apply_ops=True)
    jb = ref.sv(6).adjoint(ops, specs, tp, apply_ops=True)
    assert_close(ja, jb, np.complex128, what="adjoint Jacobian")


def _vjp_circuit(rng, n):
    # parametric gates of several generator kinds (plain, two-wire, multi-wire,
    # controlled by name and by control wires), some inverted, plus CNOTs
    ops = []
    for layer in range(3):
        for q in range(n):
            name = str(rng.choice(["RX", "RY", "RZ", "PhaseShift"]))
            ops.append(dict(name=name, wires=[q], params=[float(rng.uniform(0, 2 * np.pi))],
                            inverse=bool(rng.integers(0, 2))))
        ops.append(dict(name="CNOT", wires=[layer % n, (layer + 1) % n]))
        ops.append(dict(name="IsingXX", wires=[0, n - 1], params=[float(rng.uniform(0, 6))]))
        ops.append(dict(name="CRY", wires=[1, 2], params=[float(rng.uniform(0, 6))], inverse=True))
        ops.append(dict(name="MultiRZ", wires=[0, 2, 3], params=[float(rng.uniform(0, 6))]))
        ops.append(dict(name="RX", wires=[3], params=[float(rng.uniform(0, 6))], cwires=[0, 4], cvals=[True, False]))
    return ops


@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
def test_restatement_vs_reference_vjp(oracle, dt):
    ref = _ref()
    rng = np.random.default_rng(seed_of("vjp-pin", dt.__name__))
    n = 5
    ops = _vjp_circuit(rng, n)
    npar = sum(1 for o in ops if o.get("params"))
    tp = sorted(int(x) for x in rng.choice(npar, size=npar // 2, replace=False))
    dy = rand_state(rng, n, np.complex128)
    wa = oracle.sv(n, dt).vjp(ops, dy, tp, apply_ops=True)
    wb = ref.sv(n, dt).vjp(ops, dy, tp, apply_ops=True)
    assert wa.shape == (len(tp),)
    assert_close(wa, wb, dt, what="VJP")


def test_vjp_restatement_matches_finite_differences(oracle):
    # w_j = <dy| d psi / d theta_j>: central differences of the state (c128)
    rng = np.random.default_rng(seed_of("vjp-fd"))
    n = 5
    ops = _vjp_circuit(rng, n)
    dy = rand_state(rng, n, np.complex128)
    pidx = [i for i, o in enumerate(ops) if o.get("params")]
    tp = [0, 3, 7, len(pidx) - 1]
    w = oracle.sv(n, np.complex128).vjp(ops, dy, tp, apply_ops=True)

    def state(shift_op, h):
        o2 = [dict(o) for o in ops]
        if shift_op is not None:
            o2[shift_op]["params"] = [o2[shift_op]["params"][0] + h]
        s = oracle.sv(n, np.complex128)
        for o in o2:
            s.apply(o["name"], o["wires"], o.get("inverse", False), o.get("params", ()), o.get("cwires", ()),
                    o.get("cvals", ()))
        return s.state()

    h = 1e-5
    for k, j in enumerate(tp):
        d = (state(pidx[j], h) - state(pidx[j], -h)) / (2 * h)
        assert abs(np.vdot(dy, d) - w[k]) < 1e-8


def test_golden_vjp_config3_small(oracle, golden):
    # the reference's VectorJacobianProduct on the reduced config-3 circuit
    from lightning_gb300.workloads import config3

    g, _ = golden
    circuit, _ = config3(8, 3, seed=1003, nterms=20)
    tp = list(range(sum(1 for op in circuit if op.params)))[::2]
    w = oracle.sv(8, np.complex128).vjp([op.as_dict() for op in circuit], g["config3_small_vjp_dy"], tp,
                                        apply_ops=True)
    assert_close(w, g["config3_small_vjp"], np.complex128, what="config-3 VJP")
