"""Generate the golden fixtures in this directory from the REFERENCE itself.

Runs lightning.qubit's own C++ (compiled from the reference checkout by
oracle/build_oracle.py into oracle/_ref/libplref.so) on seeded inputs and
stores the outputs in ``golden_lq.npz``.  Only this script needs the reference
checkout; the fixtures travel with the repository, so tests on any machine
can compare both the CPU restatement and the GPU backend against them.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path[:0] = [str(REPO), str(REPO / "tests"), str(REPO / "pennylane-lightning_gb300")]

from gate_table import CONTROLLED_GATES, CONTROLLED_GENERATORS, GATES, GENERATORS, gate_params, gate_wires  # noqa: E402
from lightning_gb300.workloads import config0, config1, config3, random_pauli_sum, sum_z  # noqa: E402
from oracle.build_oracle import build_reference  # noqa: E402
from oracle.pyoracle import Oracle, pauli_sum_spec  # noqa: E402

OUT = HERE / "golden_lq.npz"


def rand_state(rng, n, dt):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return (v / np.linalg.norm(v)).astype(dt)


def main() -> int:
    if build_reference() is None:
        print("reference checkout not available; fixtures unchanged")
        return 1
    ref = Oracle("ref")
    rng = np.random.default_rng(20261203)
    arrays: dict[str, np.ndarray] = {}
    meta: dict[str, dict] = {}
    n = 5
    for dt, tag in ((np.complex128, "c128"), (np.complex64, "c64")):
        st = rand_state(rng, n, dt)
        arrays[f"state_in_{tag}"] = st
        for name in sorted(GATES):
            for inv in (False, True):
                w = gate_wires(name, rng, n)
                p = gate_params(name, rng)
                s = ref.sv(n, dt)
                s.set_state(st)
                s.apply(name, w, inv, p)
                key = f"gate_{tag}_{name}_{int(inv)}"
                arrays[key] = s.state()
                meta[key] = {"wires": w, "params": p, "inverse": inv}
        for name in CONTROLLED_GATES:
            nwk = GATES[name][0] or 2
            ws = [int(x) for x in rng.choice(n, size=nwk + 2, replace=False)] if nwk + 2 <= n else None
            if ws is None:
                continue
            cv = [bool(x) for x in rng.integers(0, 2, size=2)]
            p = gate_params(name, rng)
            s = ref.sv(n, dt)
            s.set_state(st)
            s.apply(name, ws[:nwk], False, p, ws[nwk:], cv)
            key = f"cgate_{tag}_{name}"
            arrays[key] = s.state()
            meta[key] = {"wires": ws[:nwk], "cwires": ws[nwk:], "cvals": cv, "params": p}
        for name in GENERATORS:
            w = gate_wires(name, rng, n)
            s = ref.sv(n, dt)
            s.set_state(st)
            sc = s.apply_generator(name, w)
            key = f"gen_{tag}_{name}"
            arrays[key] = s.state()
            meta[key] = {"wires": w, "scale": sc}
        for name in CONTROLLED_GENERATORS:
            nwk = GATES[name][0] or 2
            if nwk + 1 > n:
                continue
            ws = [int(x) for x in rng.choice(n, size=nwk + 1, replace=False)]
            cv = [bool(rng.integers(0, 2))]
            s = ref.sv(n, dt)
            s.set_state(st)
            sc = s.apply_generator(name, ws[:nwk], False, ws[nwk:], cv)
            key = f"cgen_{tag}_{name}"
            arrays[key] = s.state()
            meta[key] = {"wires": ws[:nwk], "cwires": ws[nwk:], "cvals": cv, "scale": sc}
        for k in (1, 2, 3):
            for inv in (False, True):
                d = 1 << k
                U = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))[0]
                w = [int(x) for x in rng.choice(n, size=k, replace=False)]
                s = ref.sv(n, dt)
                s.set_state(st)
                s.apply_matrix(U, w, inv)
                key = f"mat_{tag}_{k}_{int(inv)}"
                arrays[key] = s.state()
                arrays[key + "_U"] = U
                meta[key] = {"wires": w, "inverse": inv}
        # measurements on the input state
        s = ref.sv(n, dt)
        s.set_state(st)
        for i, wires in enumerate([None, [0], [4], [3, 1], [1, 3], [4, 0, 2], [2, 3, 0, 4, 1], [0, 1, 2, 3, 4]]):
            key = f"probs_{tag}_{i}"
            arrays[key] = s.probs(wires)
            meta[key] = {"wires": wires}
        for name in ("PauliX", "PauliY", "PauliZ", "Hadamard"):
            vals = [s.expval_named(name, [w]) for w in range(n)]
            arrays[f"expval_{tag}_{name}"] = np.array(vals)
        terms = random_pauli_sum(rng, n, 12).terms()
        spec = pauli_sum_spec(terms)
        arrays[f"ham_{tag}"] = np.array([s.expval_obs(spec), s.var_obs(spec)])
        meta[f"ham_{tag}"] = {"terms": [[c, wd, ws] for c, wd, ws in terms]}
        arrays[f"samples_{tag}"] = s.samples(2000, 37)
        arrays[f"samples_w_{tag}"] = s.samples(2000, 37, [3, 0])
        # Metropolis-Hastings samples for both transition-kernel names
        for kname in ("Local", "NonZeroRandom"):
            arrays[f"mcmc_{kname}_{tag}"] = s.mcmc_samples(kname, 50, 1500, 91)

    # config 0 (reduced n and full n = 20), c128
    for nq, layers, tag in ((8, 3, "small"), (20, 10, "full")):
        circuit = config0(nq, layers, seed=1000)
        s = ref.sv(nq, np.complex128)
        for op in circuit:
            s.apply(op.name, op.wires, False, op.params)
        spec = pauli_sum_spec(sum_z(nq).terms())
        st = s.state()
        idx = np.random.default_rng(7).choice(1 << nq, size=min(1 << nq, 512), replace=False)
        arrays[f"config0_{tag}_idx"] = idx
        arrays[f"config0_{tag}_amps"] = st[idx]
        arrays[f"config0_{tag}_expval"] = np.array([s.expval_obs(spec)])
        tp = list(range(sum(1 for o in circuit if o.params)))
        jac = ref.sv(nq, np.complex128).adjoint([o.as_dict() for o in circuit], [spec], tp, apply_ops=True)
        arrays[f"config0_{tag}_jac"] = jac[0]
        meta[f"config0_{tag}"] = {"n": nq, "layers": layers, "seed": 1000}

    # config 1 (reduced): dense SU(2) + CZ, 64-term Hamiltonian
    circuit, ham = config1(12, 4, seed=1001)
    s = ref.sv(12, np.complex128)
    for op in circuit:
        if op.matrix is not None:
            s.apply_matrix(op.matrix, op.wires, False)
        else:
            s.apply(op.name, op.wires, False, op.params)
    arrays["config1_small_state"] = s.state()
    arrays["config1_small_expval"] = np.array([s.expval_obs(pauli_sum_spec(ham.terms()))])
    meta["config1_small"] = {"n": 12, "cycles": 4, "seed": 1001}

    # config 3 (reduced): strongly entangling ansatz, Pauli Hamiltonian
    circuit, ham = config3(8, 3, seed=1003, nterms=20)
    tp = list(range(sum(1 for o in circuit if o.params)))
    jac = ref.sv(8, np.complex128).adjoint([o.as_dict() for o in circuit], [pauli_sum_spec(ham.terms())], tp,
                                           apply_ops=True)
    arrays["config3_small_jac"] = jac[0]
    meta["config3_small"] = {"n": 8, "layers": 3, "seed": 1003, "nterms": 20}
    # VectorJacobianProduct on the same circuit: seeded cotangent, every other parameter
    dy = rand_state(np.random.default_rng(1005), 8, np.complex128)
    tpv = tp[::2]
    arrays["config3_small_vjp_dy"] = dy
    arrays["config3_small_vjp"] = ref.sv(8, np.complex128).vjp([o.as_dict() for o in circuit], dy, tpv,
                                                               apply_ops=True)
    meta["config3_small_vjp"] = {"dy_seed": 1005, "trainable": "every other parameter"}

    arrays["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({OUT.stat().st_size / 1024:.0f} KiB, {len(arrays)} arrays)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
