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
