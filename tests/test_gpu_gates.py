"""GPU gate kernels vs the CPU oracle, every gate, both precisions.

Pattern of the reference's kernel-comparison tests
(pennylane_lightning/core/simulators/lightning_qubit/gates/tests/
Test_GateImplementations_CompareKernels.cpp:168-342): random normalized states,
random wires, every gate / controlled gate / generator, compared element-wise.
"""
import itertools

import numpy as np
import pytest

from gate_table import CONTROLLED_GATES, CONTROLLED_GENERATORS, GATES, GENERATORS, gate_params, gate_wires
from helpers import DTYPES, assert_close, rand_state, rand_unitary, seed_of, sv_class

pytestmark = pytest.mark.gpu


def _pair(ops, oracle, n, dt, st):
    sv = sv_class(ops, dt)(n)
    sv.updateData(st)
    o = oracle.sv(n, dt)
    o.set_state(st)
    return sv, o


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("inverse", [False, True])
@pytest.mark.parametrize("name", sorted(GATES))
def test_named_gate(ops_module, oracle, name, inverse, dt):
    rng = np.random.default_rng(seed_of("gate", name, inverse, dt.__name__))
    for n in (4, 9, 13):
        st = rand_state(rng, n, dt)
        w = gate_wires(name, rng, n)
        p = gate_params(name, rng)
        sv, o = _pair(ops_module, oracle, n, dt, st)
        getattr(sv, name)(w, inverse, p)
        o.apply(name, w, inverse, p)
        assert_close(sv.state(), o.state(), dt, what=f"{name} n={n} w={w}")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("name", ["PauliX", "Hadamard", "RX", "RY", "RZ", "Rot", "PhaseShift", "S", "T", "SX"])
def test_one_wire_every_wire(ops_module, oracle, name, dt):
    # every target bit, including bit 0 (the last wire: adjacent amplitudes)
    rng = np.random.default_rng(seed_of("every", name, dt.__name__))
    n = 8
    st = rand_state(rng, n, dt)
    sv, o = _pair(ops_module, oracle, n, dt, st)
    for w in range(n):
        p = gate_params(name, rng)
        getattr(sv, name)([w], False, p)
        o.apply(name, [w], False, p)
    assert_close(sv.state(), o.state(), dt, what=name)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("name", ["CNOT", "CZ", "SWAP", "IsingXY", "CRY", "SingleExcitation", "IsingZZ"])
def test_two_wire_every_pair(ops_module, oracle, name, dt):
    rng = np.random.default_rng(seed_of("pairs", name, dt.__name__))
    n = 5
    st = rand_state(rng, n, dt)
    sv, o = _pair(ops_module, oracle, n, dt, st)
    for a, b in itertools.permutations(range(n), 2):
        p = gate_params(name, rng)
        getattr(sv, name)([a, b], False, p)
        o.apply(name, [a, b], False, p)
    assert_close(sv.state(), o.state(), dt, what=name)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("inverse", [False, True])
@pytest.mark.parametrize("name", CONTROLLED_GATES)
def test_controlled_gate(ops_module, oracle, name, inverse, dt):
    rng = np.random.default_rng(seed_of("cgate", name, inverse, dt.__name__))
    n = 8
    nwk = GATES[name][0] or 2
    for nc in (1, 2, 3):
        st = rand_state(rng, n, dt)
        ws = [int(x) for x in rng.choice(n, size=nwk + nc, replace=False)]
        w, cw = ws[:nwk], ws[nwk:]
        cv = [bool(x) for x in rng.integers(0, 2, size=nc)]
        p = gate_params(name, rng)
        sv, o = _pair(ops_module, oracle, n, dt, st)
        getattr(sv, name)(cw, cv, w, inverse, p)
        o.apply(name, w, inverse, p, cw, cv)
        assert_close(sv.state(), o.state(), dt, what=f"C-{name} cw={cw} cv={cv}")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("name", GENERATORS)
def test_generator(ops_module, oracle, name, dt):
    rng = np.random.default_rng(seed_of("gen", name, dt.__name__))
    n = 7
    st = rand_state(rng, n, dt)
    w = gate_wires(name, rng, n)
    sv, o = _pair(ops_module, oracle, n, dt, st)
    s1 = sv.applyGenerator(name, w)
    s2 = o.apply_generator(name, w)
    assert s1 == s2
    assert_close(sv.state(), o.state(), dt, what=f"gen {name}")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("name", CONTROLLED_GENERATORS)
def test_controlled_generator(ops_module, oracle, name, dt):
    rng = np.random.default_rng(seed_of("cgen", name, dt.__name__))
    n = 8
    nwk = GATES[name][0] or 2
    st = rand_state(rng, n, dt)
    ws = [int(x) for x in rng.choice(n, size=nwk + 2, replace=False)]
    w, cw = ws[:nwk], ws[nwk:]
    cv = [bool(x) for x in rng.integers(0, 2, size=2)]
    sv, o = _pair(ops_module, oracle, n, dt, st)
    s1 = sv.applyGenerator(name, w, False, cw, cv)
    s2 = o.apply_generator(name, w, False, cw, cv)
    assert s1 == s2
    assert_close(sv.state(), o.state(), dt, what=f"cgen {name}")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("inverse", [False, True])
def test_apply_matrix(ops_module, oracle, k, inverse, dt):
    rng = np.random.default_rng(seed_of("mat", k, inverse, dt.__name__))
    n = 9
    for nc in (0, 2):
        st = rand_state(rng, n, dt)
        ws = [int(x) for x in rng.choice(n, size=k + nc, replace=False)]
        w, cw = ws[:k], ws[k:]
        cv = [bool(x) for x in rng.integers(0, 2, size=nc)]
        U = rand_unitary(rng, k)
        sv, o = _pair(ops_module, oracle, n, dt, st)
        if nc:
            sv.applyControlledMatrix(U, cw, cv, w, inverse)
        else:
            sv.applyMatrix(U, w, inverse)
        o.apply_matrix(U, w, inverse, cw, cv)
        assert_close(sv.state(), o.state(), dt, what=f"matrix k={k} nc={nc}")


@pytest.mark.parametrize("dt", DTYPES)
def test_apply_sparse_matrix(ops_module, oracle, dt):
    rng = np.random.default_rng(seed_of("sparse-op", dt.__name__))
    n, k = 7, 3
    st = rand_state(rng, n, dt)
    U = rand_unitary(rng, k)
    U[np.abs(U) < 0.3] = 0
    rows, cols = np.nonzero(U)
    indptr = np.searchsorted(rows, np.arange((1 << k) + 1))
    data = U[rows, cols]
    w = [5, 1, 3]
    sv, o = _pair(ops_module, oracle, n, dt, st)
    sv.applySparseMatrix(indptr, cols, data, w)
    o.apply_sparse(indptr, cols, data, w)
    assert_close(sv.state(), o.state(), dt, what="sparse op")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("word", ["X", "Y", "Z", "XY", "ZZ", "XYZ", "YIZX", "ZZZZ"])
@pytest.mark.parametrize("inverse", [False, True])
def test_pauli_rot(ops_module, oracle, word, inverse, dt):
    rng = np.random.default_rng(seed_of("prot", word, inverse, dt.__name__))
    n = 8
    st = rand_state(rng, n, dt)
    w = [int(x) for x in rng.choice(n, size=len(word), replace=False)]
    th = float(rng.uniform(0, 6.28))
    sv, o = _pair(ops_module, oracle, n, dt, st)
    sv.applyPauliRot(w, inverse, [th], word)
    o.apply_pauli_rot(w, inverse, th, word)
    assert_close(sv.state(), o.state(), dt, what=f"PauliRot {word}")


@pytest.mark.parametrize("dt", DTYPES)
def test_state_management(ops_module, oracle, dt):
    rng = np.random.default_rng(seed_of("state", dt.__name__))
    n = 6
    SV = sv_class(ops_module, dt)
    sv = SV(n)
    assert len(sv) == 64 and sv.size() == 64
    e0 = np.zeros(64, dt)
    e0[0] = 1
    assert np.array_equal(sv.state(), e0)
    sv.setBasisState([1, 0, 1], [0, 3, 5])
    o = oracle.sv(n, dt)
    o.set_basis_state([1, 0, 1], [0, 3, 5])
    assert np.array_equal(sv.state(), o.state())
    sub = rand_state(rng, 3, dt)
    sv.setStateVector(sub, [4, 0, 2])
    ref = np.zeros(64, dt)
    for j in range(8):
        idx = (((j >> 2) & 1) << (n - 1 - 4)) | (((j >> 1) & 1) << (n - 1 - 0)) | ((j & 1) << (n - 1 - 2))
        ref[idx] = sub[j]
    assert np.array_equal(sv.state(), ref)
    st = rand_state(rng, n, dt)
    sv.updateData(st)
    o.set_state(st)
    sv.collapse(2, True)
    o.collapse(2, True)
    assert_close(sv.state(), o.state(), dt, what="collapse")
    sv.resetStateVector()
    assert np.array_equal(sv.state(), e0)


def test_errors(ops_module):
    sv = ops_module.StateVectorC128(4)
    with pytest.raises(RuntimeError, match="disjoint"):
        sv.CNOT([1, 1], False, [])
    with pytest.raises(RuntimeError):
        sv.RX([7], False, [0.1])
    with pytest.raises(RuntimeError, match="size of matrix"):
        sv.applyMatrix(np.eye(4), [0], False)
    with pytest.raises(RuntimeError, match="not supported"):
        sv.applyOperation("NoSuchGate", [0], False, [])
    sv.updateData(np.zeros(16, np.complex128))
    with pytest.raises(RuntimeError, match="norm close to zero"):
        sv.normalize()
