"""GPU backend vs the golden fixtures produced by the reference's own C++
(tests/golden/make_golden.py): per-gate states, probabilities (bit-exact for
all wires), expectation values, seeded and Metropolis-Hastings samples
(exact), and config 0 at its
full size (20 qubits, 10 layers: <sum Z> and the 600-parameter Jacobian).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import assert_close, assert_scalar, meas_class, obs_ns, sv_class

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_lq.npz"
DT = {"c128": np.complex128, "c64": np.complex64}


@pytest.fixture(scope="module")
def golden():
    g = np.load(GOLDEN)
    return g, json.loads(str(g["meta"]))


@pytest.mark.parametrize("tag", ["c128", "c64"])
def test_gates_vs_reference(ops_module, golden, tag):
    g, meta = golden
    dt = DT[tag]
    st = g[f"state_in_{tag}"]
    SV = sv_class(ops_module, dt)
    for key, m in meta.items():
        kind = key.split("_")[0]
        if kind not in ("gate", "cgate", "gen", "cgen", "mat") or key.split("_")[1] != tag:
            continue
        sv = SV(5)
        sv.updateData(st)
        name = key.split("_")[2]
        if kind == "gate":
            getattr(sv, name)(m["wires"], m["inverse"], m["params"])
        elif kind == "cgate":
            getattr(sv, name)(m["cwires"], m["cvals"], m["wires"], False, m["params"])
        elif kind == "gen":
            assert sv.applyGenerator(name, m["wires"]) == m["scale"]
        elif kind == "cgen":
            assert sv.applyGenerator(name, m["wires"], False, m["cwires"], m["cvals"]) == m["scale"]
        else:
            sv.applyMatrix(g[key + "_U"], m["wires"], m["inverse"])
        assert_close(sv.state(), g[key], dt, what=key)


@pytest.mark.parametrize("tag", ["c128", "c64"])
def test_measurements_vs_reference(ops_module, golden, tag):
    g, meta = golden
    dt = DT[tag]
    sv = sv_class(ops_module, dt)(5)
    sv.updateData(g[f"state_in_{tag}"])
    m = meas_class(ops_module, dt)(sv)
    # full distribution: element-wise, bit-exact with the reference
    assert np.array_equal(m.probs(), g[f"probs_{tag}_0"].astype(m.probs().dtype))
    for i in range(1, 8):
        assert_close(m.probs(meta[f"probs_{tag}_{i}"]["wires"]), g[f"probs_{tag}_{i}"], dt, what=f"probs {i}")
    for name in ("PauliX", "PauliY", "PauliZ", "Hadamard"):
        for w in range(5):  # one-wire observables have norm 1
            assert_scalar(m.expval(name, [w]), g[f"expval_{tag}_{name}"][w], dt, mag=1.0, what=f"E {name}{w}")
    Named, _, Prod, Ham, _ = obs_ns(ops_module, dt)
    names = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}
    terms = meta[f"ham_{tag}"]["terms"]
    H = Ham([t[0] for t in terms], [Prod([Named(names[c], [w]) for c, w in zip(t[1], t[2])]) for t in terms])
    c1 = sum(abs(t[0]) for t in terms)  # error scale of a Pauli-sum expectation (and its square for var)
    assert_scalar(m.expval(H), g[f"ham_{tag}"][0], dt, mag=c1, what="E ham")
    assert_scalar(m.var(H), g[f"ham_{tag}"][1], dt, mag=c1 * c1, what="V ham")
    m.set_random_seed(37)
    assert np.array_equal(m.generate_samples(5, 2000).astype(np.int64), g[f"samples_{tag}"])
    assert np.array_equal(m.generate_samples([3, 0], 2000).astype(np.int64), g[f"samples_w_{tag}"])
    m.set_random_seed(91)
    for kname in ("Local", "NonZeroRandom"):
        s = m.generate_mcmc_samples(5, kname, 50, 1500).astype(np.int64)
        assert np.array_equal(s, g[f"mcmc_{kname}_{tag}"]), kname


@pytest.mark.parametrize("size", ["small", "full"])
def test_config0_vs_reference(ops_module, golden, size):
    from lightning_gb300.workloads import config0

    g, meta = golden
    n, layers = meta[f"config0_{size}"]["n"], meta[f"config0_{size}"]["layers"]
    circuit = config0(n, layers, seed=1000)
    sv = ops_module.StateVectorC128(n)
    for op in circuit:
        getattr(sv, op.name)(op.wires, False, op.params)
    st = sv.state()
    assert_close(st[g[f"config0_{size}_idx"]], g[f"config0_{size}_amps"], np.complex128, what="state")
    Named, _, _, Ham, _ = obs_ns(ops_module, np.complex128)
    H = Ham([1.0] * n, [Named("PauliZ", [q]) for q in range(n)])
    e = ops_module.MeasurementsC128(sv).expval(H)
    # <sum Z> cancels (about 1e-3 at 20 qubits from n terms of norm 1): its
    # error is relative to sum |c| = n
    assert_scalar(e, g[f"config0_{size}_expval"][0], np.complex128, mag=float(n), what="<sum Z>")
    ops = ops_module.OpsStructC128([o.name for o in circuit], [o.params for o in circuit],
                                   [o.wires for o in circuit], [False] * len(circuit), [None] * len(circuit))
    tp = list(range(sum(1 for o in circuit if o.params)))
    jac = ops_module.AdjointJacobianC128()(ops_module.StateVectorC128(n), [H], ops, tp, True)
    ref = g[f"config0_{size}_jac"]
    assert_close(jac, ref, np.complex128, what="config-0 Jacobian")


def test_config1_config3_small_vs_reference(ops_module, golden):
    from lightning_gb300.workloads import config1, config3

    g, _ = golden
    circuit, ham = config1(12, 4, seed=1001)
    sv = ops_module.StateVectorC128(12)
    for op in circuit:
        if op.matrix is not None:
            sv.applyMatrix(op.matrix, op.wires, False)
        else:
            getattr(sv, op.name)(op.wires, False, op.params)
    assert_close(sv.state(), g["config1_small_state"], np.complex128, what="config1")
    Named, _, Prod, Ham, _ = obs_ns(ops_module, np.complex128)
    names = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}
    H = Ham(ham.coeffs, [Prod([Named(names[c], [w]) for c, w in zip(wd, ws)]) for wd, ws in zip(ham.words, ham.wires)])
    assert_scalar(ops_module.MeasurementsC128(sv).expval(H), g["config1_small_expval"][0], np.complex128,
                  mag=float(np.sum(np.abs(ham.coeffs))), what="config-1 <H>")
    circuit, ham = config3(8, 3, seed=1003, nterms=20)
    H = Ham(ham.coeffs, [Prod([Named(names[c], [w]) for c, w in zip(wd, ws)]) for wd, ws in zip(ham.words, ham.wires)])
    ops = ops_module.OpsStructC128([o.name for o in circuit], [o.params for o in circuit],
                                   [o.wires for o in circuit], [False] * len(circuit), [None] * len(circuit))
    tp = list(range(sum(1 for o in circuit if o.params)))
    jac = ops_module.AdjointJacobianC128()(ops_module.StateVectorC128(8), [H], ops, tp, True)
    assert_close(jac, g["config3_small_jac"], np.complex128, what="config-3 Jacobian")
