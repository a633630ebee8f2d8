"""Batch engine (plgb_batch_*): many circuits in one run vs the CPU oracle.

Every circuit of a batch starts from |0...0>; its Pauli-sum expectation
values must match the oracle applying the same gates one by one, within
1e-12 (complex128) / 1e-5 (complex64) relative to max(1, |value|) times the
observable's coefficient norm.  A circuit's values must be bit-identical
alone and inside any batch, and across wave splits.
"""
from types import SimpleNamespace

import numpy as np
import pytest

from gate_table import GATES, gate_params
from helpers import DTYPES, assert_close, assert_scalar, seed_of
from lightning_gb300.batch import BatchEngine, pack
from lightning_gb300.workloads import Op, PauliSum, config0, config2_packed, random_pauli_sum, sum_z

pytestmark = pytest.mark.gpu

PREC = {np.complex128: 128, np.complex64: 64}


def named_circuit(rng, n, depth):
    """Random named gates of every family on at most 4 wires."""
    ops = []
    # PCPhase's dimension check depends on the register size: keep it to n >= 2
    names = [g for g in GATES if (GATES[g][0] or 1) <= min(4, n) and g not in ("Identity",)
             and not (g == "PCPhase" and n < 2)]
    for _ in range(depth):
        name = str(rng.choice(names))
        nw = GATES[name][0] or int(rng.integers(1, min(4, n) + 1))
        w = [int(x) for x in rng.choice(n, size=nw, replace=False)]
        ops.append(Op(name, w, [float(p) for p in gate_params(name, rng)], inverse=bool(rng.integers(0, 2))))
    return ops


def oracle_values(oracle, dt, circ):
    from oracle.pyoracle import pauli_sum_spec

    o = oracle.sv(circ.n, dt)
    st = np.zeros(1 << circ.n, dt)
    st[0] = 1
    o.set_state(st)
    for op in circ.ops:
        o.apply(op.name, op.wires, op.inverse, op.params)
    return np.array([o.expval_obs(pauli_sum_spec(obs.terms())) for obs in circ.observables])


def check(values, ref, circs, dt, what):
    # each expectation value relative to its natural size sum |c| (Pauli
    # words have norm 1): <sum Z> and short Pauli sums can cancel to ~0
    k = 0
    for c in circs:
        for obs in c.observables:
            c1 = float(np.sum(np.abs(obs.coeffs)))
            assert_scalar(values[k], ref[k], dt, mag=c1, what=f"{what}: observable {k}")
            k += 1


def mixed_batch(seed, sizes, depth=30):
    rng = np.random.default_rng(seed)
    circs = []
    for n in sizes:
        obs = [sum_z(n), random_pauli_sum(rng, n, 5, 1, min(4, n)), random_pauli_sum(rng, n, 1, min(2, n), min(2, n))]
        circs.append(SimpleNamespace(n=n, ops=named_circuit(rng, n, depth), observables=obs))
    return circs


@pytest.mark.parametrize("dt", DTYPES)
def test_batch_named_gates_vs_oracle(oracle, dt):
    # sizes below 9 run padded; sizes 9..14 span one to many tiles
    circs = mixed_batch(seed_of("batch", dt.__name__), [1, 2, 3, 5, 8, 9, 10, 11, 12, 13, 14])
    eng = BatchEngine(PREC[dt])
    vals = eng.run(pack(circs))
    ref = np.concatenate([oracle_values(oracle, dt, c) for c in circs])
    check(vals, ref, circs, dt, "named gates")
    st = eng.stats()
    assert st["circuits"] == len(circs) and st["padded"] == 5 and st["launches"] >= 2


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("tile_bits", [9, 10, 12])
def test_batch_config0_fixed_tiles(oracle, dt, tile_bits):
    rng = np.random.default_rng(seed_of("batch-c0", tile_bits))
    circs = []
    for n in (9, 12, 15):
        circs.append(SimpleNamespace(n=n, ops=config0(n, 3, seed=int(rng.integers(1 << 30))),
                                     observables=[sum_z(n), random_pauli_sum(rng, n, 3, 2, 2)]))
    vals = BatchEngine(PREC[dt], tile_bits=tile_bits).run(pack(circs))
    ref = np.concatenate([oracle_values(oracle, dt, c) for c in circs])
    check(vals, ref, circs, dt, f"config0 t={tile_bits}")


@pytest.mark.parametrize("dt", DTYPES)
def test_batch_alone_equals_mixed(dt):
    packed = config2_packed(24, seed=77)
    eng = BatchEngine(PREC[dt])
    mixed = packed.observables_of(eng.run(packed))
    for c in (0, 5, 17, 23):
        alone = eng.run(packed.select([c]))
        assert np.array_equal(alone, mixed[c]), f"circuit {c}: alone {alone} vs mixed {mixed[c]}"
    # reversed order gives the same bits
    rev = list(range(packed.num_circuits))[::-1]
    again = eng.run(packed.select(rev))
    for i, c in enumerate(rev):
        assert np.array_equal(again[4 * i:4 * i + 4], mixed[c])
    # so does a second engine with the same tile sizes (autotuning may pick
    # other sizes, which round differently)
    a = BatchEngine(PREC[dt], tile_bits=10).run(packed)
    b = BatchEngine(PREC[dt], tile_bits=10).run(packed.select(rev))
    for i, c in enumerate(rev):
        assert np.array_equal(b[4 * i:4 * i + 4], a[4 * c:4 * c + 4])


@pytest.mark.parametrize("dt", DTYPES)
def test_batch_waves_equal_single_wave(dt):
    packed = config2_packed(12, seed=5)
    one = BatchEngine(PREC[dt], tile_bits=11).run(packed)
    eng = BatchEngine(PREC[dt], tile_bits=11, wave_bytes=1)  # one register per wave
    many = eng.run(packed)
    assert np.array_equal(one, many)
    st = eng.stats()
    assert st["waves"] == packed.num_circuits and st["wave_of"] == list(range(packed.num_circuits))


def test_batch_config2_sample_vs_oracle(oracle):
    packed = config2_packed(4096, seed=1002)
    idx = [0, 1, 2, 3]
    sub = packed.select(idx)
    vals = BatchEngine(128).run(sub)
    from lightning_gb300.workloads import config2

    circs = [SimpleNamespace(n=c.n, ops=c.ops, observables=c.observables) for c in config2(4, seed=1002)]
    ref = np.concatenate([oracle_values(oracle, np.complex128, c) for c in circs])
    check(vals, ref, circs, np.complex128, "config2 sample")


def test_batch_edge_cases(oracle):
    eng = BatchEngine(128)
    # empty batch
    empty = pack([])
    assert eng.run(empty).shape == (0,)
    # a circuit without gates, one without observables, an observable with no terms
    circs = [SimpleNamespace(n=4, ops=[], observables=[sum_z(4)]),
             SimpleNamespace(n=6, ops=[Op("Hadamard", [0])], observables=[]),
             SimpleNamespace(n=3, ops=[Op("PauliX", [1])], observables=[PauliSum([], [], []), sum_z(3)])]
    vals = eng.run(pack(circs))
    assert np.allclose(vals, [4.0, 0.0, 1.0], atol=1e-12)


def test_batch_rejects_bad_input():
    from lightning_gb300._capi import LightningException

    eng = BatchEngine(128)
    bad = pack([SimpleNamespace(n=3, ops=[Op("RX", [5], [0.1])], observables=[])])
    with pytest.raises(LightningException, match="wire index out of range"):
        eng.run(bad)
    with pytest.raises(ValueError):
        pack([SimpleNamespace(n=3, ops=[Op("QubitUnitary", [0], matrix=np.eye(2))], observables=[])])


def test_batch_double_float_vs_fp64(ops_module):
    # complex128 batches run in FP64 by default; the opt-in double-float
    # passes give the same values within the complex128 tolerance, relative
    # to each expectation value's natural size sum |c|
    packed = config2_packed(10, seed=21)
    b = BatchEngine(128, tile_bits=10)
    vb = b.run(packed)
    assert b.stats()["double_float"] is False
    prev = ops_module.set_c128_fp64_passes(False)
    try:
        a = BatchEngine(128, tile_bits=10)
        va = a.run(packed)
        assert a.stats()["double_float"] is True
    finally:
        ops_module.set_c128_fp64_passes(prev)
    for k in range(packed.num_observables):
        c1 = float(np.abs(packed.term_coeffs[packed.term_offsets[k]:packed.term_offsets[k + 1]]).sum())
        assert_scalar(va[k], vb[k], np.complex128, mag=c1, what=f"observable {k}")


def test_batch_adjoint_matches_single_register_adjoint(ops_module):
    # run_adjoint == <H> and AdjointJacobianC128 of each circuit alone
    from lightning_gb300.workloads import config4_packed

    packed, _, _ = config4_packed(rate=2000.0, duration=0.01, seed=9, n_max=11)
    eng = BatchEngine(128)
    vals, jacs = eng.run_adjoint(packed)
    from lightning_gb300.serve import Server

    srv = Server(128, adjoint_lanes=1)
    srv.packed, srv.adjoint = packed, np.ones(packed.num_circuits, bool)
    for c in range(0, packed.num_circuits, 3):
        n = int(packed.num_qubits[c])
        S = srv._ops_struct(c)
        H = srv._hamiltonian(c)
        sv = ops_module.StateVectorC128(n)
        for name, w, prm in zip(S.names, S.wires, S.params):
            sv.applyOperation(name, w, False, prm)
        v = float(ops_module.MeasurementsC128(sv).expval(H))
        npar = sum(1 for p in S.params if p)
        j = ops_module.AdjointJacobianC128()(sv, [H], S, list(range(npar)))
        c1 = float(np.sum(np.abs(packed.term_coeffs[packed.term_offsets[c]:packed.term_offsets[c + 1]])))
        assert_scalar(vals[c], v, np.complex128, mag=c1, what=f"<H> request {c}")  # error scale: sum |c|
        assert jacs[c].shape == (1, npar)
        assert_close(jacs[c][0], j, np.complex128, what=f"Jacobian request {c}")
        # alone (a batch of one) is bit-identical to the batch
        va, ja = srv.adjoint_one(c)
        assert va == vals[c] and np.array_equal(ja, jacs[c][0])
