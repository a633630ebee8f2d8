"""Fused tile passes vs the CPU oracle and vs the unfused per-gate path.

Random circuits mixing every gate family (one-wire named gates, controlled
gates with local and global controls, dense matrices on 1-4 wires, diagonal
and parity gates, Pauli rotations, excitations) are applied through
StateVector.applyOperations with tile sizes from 2^2 to 2^14 amplitudes.
"""
import numpy as np
import pytest

from gate_table import GATES, gate_params
from helpers import DTYPES, assert_close, rand_state, rand_unitary, rel_errors, seed_of, sv_class
from lightning_gb300.workloads import config0, config1

pytestmark = pytest.mark.gpu


def random_circuit(rng, n, depth):
    ops = []
    names = [g for g in GATES if g not in ("Identity",)]
    for _ in range(depth):
        r = rng.random()
        if r < 0.15:
            k = int(rng.integers(1, min(4, n) + 1))
            w = [int(x) for x in rng.choice(n, size=k, replace=False)]
            ops.append(dict(name="QubitUnitary", wires=w, matrix=rand_unitary(rng, k)))
        elif r < 0.25 and n >= 3:
            name = str(rng.choice(["RX", "RY", "RZ", "PhaseShift", "Hadamard", "PauliX", "Rot", "IsingXY", "MultiRZ"]))
            nwk = GATES[name][0] or 2
            nc = int(rng.integers(1, 3))
            if nwk + nc > n:
                continue
            ws = [int(x) for x in rng.choice(n, size=nwk + nc, replace=False)]
            ops.append(dict(name=name, wires=ws[:nwk], params=gate_params(name, rng), cwires=ws[nwk:],
                            cvals=[bool(x) for x in rng.integers(0, 2, size=nc)], inverse=bool(rng.integers(0, 2))))
        else:
            name = str(rng.choice(names))
            nwk = GATES[name][0] or int(rng.integers(1, min(4, n) + 1))
            if nwk > n:
                continue
            w = [int(x) for x in rng.choice(n, size=nwk, replace=False)]
            ops.append(dict(name=name, wires=w, params=gate_params(name, rng), inverse=bool(rng.integers(0, 2))))
    return ops


def ops_struct(ops_module, dt, ops):
    OS = ops_module.OpsStructC128 if np.dtype(dt) == np.complex128 else ops_module.OpsStructC64
    return OS([o["name"] for o in ops], [o.get("params", []) for o in ops], [o["wires"] for o in ops],
              [o.get("inverse", False) for o in ops], [o.get("matrix") for o in ops],
              [o.get("cwires", []) for o in ops], [o.get("cvals", []) for o in ops])


def oracle_apply(oracle, n, dt, st, ops):
    o = oracle.sv(n, dt)
    o.set_state(st)
    for op in ops:
        if op.get("matrix") is not None:
            o.apply_matrix(op["matrix"], op["wires"], op.get("inverse", False), op.get("cwires", ()),
                           op.get("cvals", ()))
        else:
            o.apply(op["name"], op["wires"], op.get("inverse", False), op.get("params", ()), op.get("cwires", ()),
                    op.get("cvals", ()))
    return o.state()


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n,tile_bits", [(4, 2), (6, 3), (8, 5), (10, 6), (12, 8), (13, 10), (14, 12), (16, 14)])
def test_random_circuits_fused(ops_module, oracle, dt, n, tile_bits):
    rng = np.random.default_rng(seed_of("fused", n, tile_bits, dt.__name__))
    ops = random_circuit(rng, n, 60)
    st = rand_state(rng, n, dt)
    sv = sv_class(ops_module, dt)(n)
    sv.updateData(st)
    passes = sv.applyOperations(ops_struct(ops_module, dt, ops), tile_bits)
    assert passes >= 1
    ref = oracle_apply(oracle, n, dt, st, ops)
    assert_close(sv.state(), ref, dt, what=f"fused n={n} t={tile_bits}")


@pytest.mark.parametrize("dt", DTYPES)
def test_fused_equals_unfused_and_cached_reuse(ops_module, dt):
    rng = np.random.default_rng(seed_of("fused-vs-unfused", dt.__name__))
    n = 11
    ops = random_circuit(rng, n, 80)
    st = rand_state(rng, n, dt)
    S = ops_struct(ops_module, dt, ops)
    a = sv_class(ops_module, dt)(n)
    b = sv_class(ops_module, dt)(n)
    a.updateData(st)
    b.updateData(st)
    a.applyOperations(S, 0)
    b.applyOperations(S, 7)
    assert_close(b.state(), a.state(), dt, what="fused vs unfused")
    # the compiled program is cached on the ops object; apply it again
    a.applyOperations(S, 0)
    b.applyOperations(S, 7)
    assert_close(b.state(), a.state(), dt, what="second application")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("tile_bits", [6, 9, 12])
def test_config1_small_fused(ops_module, oracle, dt, tile_bits):
    # dense Haar SU(2) + CZ: exercises the D.R.D rewrite, merged diagonals and
    # CZ sign flips across the tile boundary
    n = 14
    circuit, _ = config1(n, 6, seed=1001)
    ops = [op.as_dict() for op in circuit]
    st = rand_state(np.random.default_rng(3), n, dt)
    sv = sv_class(ops_module, dt)(n)
    sv.updateData(st)
    sv.applyOperations(ops_struct(ops_module, dt, ops), tile_bits)
    ref = oracle_apply(oracle, n, dt, st, ops)
    assert_close(sv.state(), ref, dt, what=f"config1 t={tile_bits}")


@pytest.mark.parametrize("dt", DTYPES)
def test_config0_fused(ops_module, oracle, dt):
    n = 12
    circuit = config0(n, 5, seed=1000)
    ops = [op.as_dict() for op in circuit]
    sv = sv_class(ops_module, dt)(n)
    sv.applyOperations(ops_struct(ops_module, dt, ops), 9)
    st = np.zeros(1 << n, dt)
    st[0] = 1
    ref = oracle_apply(oracle, n, dt, st, ops)
    assert_close(sv.state(), ref, dt, what="config0 fused")


def test_c128_double_float_passes_match_fp64(ops_module):
    # fused complex128 passes run in FP64 by default; the opt-in
    # double-float passes must agree within the complex128 tolerance
    rng = np.random.default_rng(seed_of("df-vs-fp64"))
    n = 16
    circuit, _ = config1(n, 12, seed=1001)
    ops = [op.as_dict() for op in circuit]  # every pass on the register kernel
    st = rand_state(rng, n, np.complex128)
    S = ops_struct(ops_module, np.complex128, ops)
    outs = {}
    for fp64 in (False, True):
        prev = ops_module.set_c128_fp64_passes(fp64)
        try:
            sv = ops_module.StateVectorC128(n)
            sv.updateData(st)
            sv.applyOperations(S, 11)
            outs[fp64] = sv.state()
        finally:
            ops_module.set_c128_fp64_passes(prev)
    # double-float keeps ~48 bits: within 1e-12 norm-relative of the FP64
    # passes; per amplitude its stated bound is 1e-10 (measured 2.8e-12 at
    # 24 qubits, test_gpu_parity_scale.py)
    nr, pr = rel_errors(outs[False], outs[True], np.complex128)
    assert nr <= 1e-12 and pr <= 1e-10, (nr, pr)
    assert not np.array_equal(outs[False], outs[True])  # the two arithmetics did run


def test_double_float_range(ops_module, oracle):
    # the double-float passes hold magnitudes below 2^128: a larger amplitude
    # becomes infinite (and NaN stays NaN) instead of a wrapped exponent; the
    # amplitudes it does not touch are unaffected
    n = 12
    rng = np.random.default_rng(seed_of("df-range"))
    st = rand_state(rng, n)
    st[5], st[9] = 1e300 + 0j, complex(np.nan, 0.0)
    ops = [dict(name="RZ", wires=[0], params=[0.7]), dict(name="RX", wires=[3], params=[0.4]),
           dict(name="PhaseShift", wires=[1], params=[1.1])]
    prev = ops_module.set_c128_fp64_passes(False)
    try:
        sv = ops_module.StateVectorC128(n)
        sv.updateData(st)
        sv.applyOperations(ops_struct(ops_module, np.complex128, ops), 11)
        out = sv.state()
    finally:
        ops_module.set_c128_fp64_passes(prev)
    hit = [5, 5 ^ 256, 9, 9 ^ 256]  # RX on wire 3 mixes amplitude bit 8
    assert not np.isfinite(out[hit]).any()
    rest = np.setdiff1d(np.arange(1 << n), hit)
    st_ok = st.copy()
    st_ok[hit] = 0.0
    ref = oracle_apply(oracle, n, np.complex128, st_ok, ops)
    assert np.max(np.abs(out[rest] - ref[rest])) <= 1e-10 * np.max(np.abs(ref))


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("fp64", [False, True])
def test_wide_local_diagonals_fused(ops_module, oracle, dt, fp64):
    # merged diagonals whose all-local factors span more than 4 bits (here
    # multi-controlled phases) are tabulated on the host; narrower ones are
    # expanded on the device from their factors: both kinds in one program,
    # for both complex128 pass kinds
    rng = np.random.default_rng(seed_of("wide-diag", dt.__name__, fp64))
    n = 13
    ops = []
    for layer in range(6):
        for q in range(n):
            ops.append(dict(name=str(rng.choice(["RX", "RY", "RZ", "PhaseShift"])), wires=[q],
                            params=[float(rng.uniform(0, 2 * np.pi))]))
        k = int(rng.integers(5, 8))
        w = [n - 9 + int(x) for x in rng.choice(9, size=k, replace=False)]  # amplitude bits 0-8: in the tile
        ops.append(dict(name=str(rng.choice(["PhaseShift", "RZ"])), wires=w[:1], params=[float(rng.uniform(0, 6))],
                        cwires=w[1:], cvals=[bool(x) for x in rng.integers(0, 2, size=k - 1)]))
        ops.append(dict(name="MultiRZ", wires=w, params=[float(rng.uniform(0, 2 * np.pi))]))
        ops.append(dict(name="IsingZZ", wires=[layer % n, (layer + 5) % n], params=[float(rng.uniform(0, 6))]))
        ops.append(dict(name="CNOT", wires=[layer % n, (layer + 1) % n]))
    st = rand_state(rng, n, dt)
    sv = sv_class(ops_module, dt)(n)
    sv.updateData(st)
    prev = ops_module.set_c128_fp64_passes(fp64)
    try:
        sv.applyOperations(ops_struct(ops_module, dt, ops), 11)
    finally:
        ops_module.set_c128_fp64_passes(prev)
    ref = oracle_apply(oracle, n, dt, st, ops)
    assert_close(sv.state(), ref, dt, what=f"wide diagonals fp64={fp64}")


def test_fp64_passes_keep_tiny_amplitudes(ops_module, oracle):
    # the default complex128 passes compute in FP64: amplitudes far below the
    # float range (1e-200) keep their relative accuracy, like the reference's
    # f64 kernels; the opt-in double-float passes flush them to zero
    n = 13
    rng = np.random.default_rng(seed_of("tiny-amps"))
    st = rand_state(rng, n) * 1e-200
    ops = [dict(name=str(rng.choice(["RX", "RY", "RZ"])), wires=[int(w)], params=[float(rng.uniform(0, 6))])
           for w in rng.integers(0, n, size=60)]
    ops += [dict(name="CNOT", wires=[0, 7]), dict(name="CZ", wires=[3, 12]), dict(name="RY", wires=[5], params=[0.3])]
    S = ops_struct(ops_module, np.complex128, ops)
    sv = ops_module.StateVectorC128(n)
    sv.updateData(st)
    assert sv.applyOperations(S, 11) >= 1
    ref = oracle_apply(oracle, n, np.complex128, st, ops)
    assert_close(sv.state(), ref, np.complex128, what="1e-200 amplitudes, FP64 passes")
    prev = ops_module.set_c128_fp64_passes(False)
    try:
        sv2 = ops_module.StateVectorC128(n)
        sv2.updateData(st)
        sv2.applyOperations(S, 11)
        assert not np.any(sv2.state())
    finally:
        ops_module.set_c128_fp64_passes(prev)
