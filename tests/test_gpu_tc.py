"""Dense complex64 gates on six wires on the tensor cores (tcgen05, FP32
operands split into three BF16 parts) against the oracle and against the
CUDA-core kernel: wires on low, high and mixed index bits, registers of 12
to 24 qubits, inverse matrices, and a run of several blocks."""
import numpy as np
import pytest

from helpers import assert_state, rand_state, rand_unitary, seed_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,wires", [
    (12, [6, 7, 8, 9, 10, 11]),        # the six lowest index bits (contiguous groups)
    (12, [0, 1, 2, 3, 4, 5]),          # the six highest bits
    (14, [13, 0, 7, 2, 11, 5]),        # mixed, unsorted
    (16, [3, 15, 9, 0, 12, 6]),
    (18, [17, 16, 1, 8, 4, 12]),
])
@pytest.mark.parametrize("inverse", [False, True])
def test_dense6_tensor_cores_vs_oracle(ops_module, oracle, n, wires, inverse):
    rng = np.random.default_rng(seed_of("tc6", n, tuple(wires), inverse))
    st = rand_state(rng, n, np.complex64)
    U = rand_unitary(rng, 6)
    sv = ops_module.StateVectorC64(n)
    sv.updateData(st)
    sv.applyMatrix(U, wires, inverse)
    o = oracle.sv(n, np.complex64)
    o.set_state(st)
    o.apply_matrix(U, wires, inverse)
    assert_state(sv.state(), o.state(), np.complex64, what=f"tensor-core block n={n} wires={wires}")


def test_dense6_tensor_cores_vs_cuda_cores(ops_module):
    # the same blocks on the CUDA-core kernel: equal within the complex64
    # tolerance, and not bit-identical (the tensor-core path did run)
    rng = np.random.default_rng(seed_of("tc6-vs-cc"))
    n = 16
    st = rand_state(rng, n, np.complex64)
    blocks = [(rand_unitary(rng, 6), [int(x) for x in rng.choice(n, size=6, replace=False)]) for _ in range(5)]
    out = {}
    for tc in (True, False):
        prev = ops_module.set_tc_dense(tc)
        try:
            sv = ops_module.StateVectorC64(n)
            sv.updateData(st)
            for U, w in blocks:
                sv.applyMatrix(U, w, False)
            out[tc] = sv.state()
        finally:
            ops_module.set_tc_dense(prev)
    assert_state(out[True], out[False], np.complex64, what="tensor cores vs CUDA cores")
    assert not np.array_equal(out[True], out[False])


@pytest.mark.parametrize("wires", [[18, 19, 20, 21, 22, 23], [0, 1, 2, 3, 4, 5], [23, 0, 11, 5, 17, 2]])
def test_dense6_tensor_cores_24_qubits(ops_module, wires):
    # 4096 tiles (many per CTA, every pipeline stage of the kernel in steady
    # state): the tensor-core result equals the CUDA-core kernel's within the
    # complex64 tolerance
    n = 24
    rng = np.random.default_rng(seed_of("tc6-24", tuple(wires)))
    st = rand_state(rng, n, np.complex64)
    U = rand_unitary(rng, 6)
    out = {}
    for tc in (True, False):
        prev = ops_module.set_tc_dense(tc)
        try:
            sv = ops_module.StateVectorC64(n)
            sv.updateData(st)
            sv.applyMatrix(U, wires, False)
            out[tc] = sv.state()
        finally:
            ops_module.set_tc_dense(prev)
    assert_state(out[True], out[False], np.complex64, what=f"24 qubits wires={wires}")
    assert not np.array_equal(out[True], out[False])
