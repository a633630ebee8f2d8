"""Dense-block fusion on the GPU (StateVector.applyOperationsBlocks):
random circuits and the config-1 circuit against the oracle, complex64
(blocks of four to six wires on the tensor cores) and complex128, every
block width."""
import numpy as np
import pytest

from helpers import DTYPES, assert_state, rand_state, seed_of, sv_class
from lightning_gb300.workloads import config1
from test_gpu_fusion import oracle_apply, ops_struct, random_circuit

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("k", [2, 3, 4, 5, 6])
def test_random_circuits_blocks(ops_module, oracle, dt, k):
    n = 14
    rng = np.random.default_rng(seed_of("gpu-blocks", k, np.dtype(dt).name))
    ops = random_circuit(rng, n, 80)
    st = rand_state(rng, n, dt)
    sv = sv_class(ops_module, dt)(n)
    sv.updateData(st)
    nk = sv.applyOperationsBlocks(ops_struct(ops_module, dt, ops), k)
    assert 0 < nk <= len(ops) * 4
    assert_state(sv.state(), oracle_apply(oracle, n, dt, st, ops), dt, what=f"blocks k={k}")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("k", [4, 6])
def test_config1_blocks(ops_module, oracle, dt, k):
    n = 16
    circuit, _ = config1(n, 8, seed=1001)
    ops = [op.as_dict() for op in circuit]
    st = np.zeros(1 << n, dt)
    st[0] = 1
    sv = sv_class(ops_module, dt)(n)
    S = ops_struct(ops_module, dt, ops)
    sv.applyOperationsBlocks(S, k)
    ref = oracle_apply(oracle, n, dt, st, ops)
    assert_state(sv.state(), ref, dt, what=f"config-1 blocks k={k}")
    # the cached block list applied again from |0...0>
    sv.resetStateVector()
    sv.applyOperationsBlocks(S, k)
    assert_state(sv.state(), ref, dt, what=f"config-1 blocks k={k}, cached")


def test_c64_large_registers_run_blocks_by_default(ops_module, oracle):
    # complex64 registers of 22 qubits and more run applyOperations and the
    # lazy per-gate queue as dense blocks (six-wire blocks on the tensor
    # cores); with the tensor cores off they take the tile passes.  All
    # three agree with the oracle's complex128 state at the complex64
    # tolerance.
    from lightning_gb300.workloads import config0

    n = 22
    circuit = config0(n, 3, seed=1000)
    ops = [op.as_dict() for op in circuit]
    S = ops_module.OpsStructC64([o["name"] for o in ops], [o.get("params", []) for o in ops],
                                [o["wires"] for o in ops], [False] * len(ops), [None] * len(ops))
    st0 = np.zeros(1 << n, np.complex128)
    st0[0] = 1
    o = oracle.sv(n, np.complex128)
    o.set_state(st0)
    for op in ops:
        o.apply(op["name"], op["wires"], False, op.get("params", ()))
    ref = o.state()
    sv = ops_module.StateVectorC64(n)
    nk = sv.applyOperations(S, 12)
    assert nk == len(S.block_plan(n, 6, False))  # the blocks path ran
    assert_state(sv.state(), ref, np.complex64, what="c64 blocks by default")
    lazy = ops_module.StateVectorC64(n)
    for op in ops:
        getattr(lazy, op["name"])(op["wires"], False, op.get("params", []))
    assert_state(lazy.state(), ref, np.complex64, what="c64 lazy queue as blocks")
    prev = ops_module.set_tc_dense(False)
    try:
        tiles = ops_module.StateVectorC64(n)
        assert tiles.applyOperations(S, 12) != nk  # tile passes
        assert_state(tiles.state(), ref, np.complex64, what="c64 tile passes")
    finally:
        ops_module.set_tc_dense(prev)
