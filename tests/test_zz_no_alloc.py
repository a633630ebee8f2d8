"""plgb_meas_expval_matrix_noalloc against plgb_meas_expval_matrix.

The allocation-free variant keeps its scratch in one fixed device array per
device; two calls in a row must both agree with the allocating entry point
(the second call reuses the array).  This file is collected last so that it
also runs after every other GPU test of the session.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import DTYPES, assert_scalar, rand_hermitian, rand_state, seed_of, sv_class
from lightning_gb300 import _capi

pytestmark = pytest.mark.gpu


def _expval(fn, sv, mat, wires):
    m = np.ascontiguousarray(np.asarray(mat, dtype=np.complex128))
    w = (C.c_int64 * len(wires))(*wires)
    out = C.c_double(np.nan)
    rc = getattr(_capi.lib(), fn)(sv._h, m.ctypes.data_as(C.POINTER(C.c_double)), w, len(wires), C.byref(out))
    return rc, out.value


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n,wires", [(3, [1]), (8, [0, 5]), (12, [7, 2, 11]), (14, [3, 13, 0, 8]),
                                     (16, [15, 4, 9, 0, 12])])
def test_noalloc_matches_allocating_entry(ops_module, dt, n, wires):
    rng = np.random.default_rng(seed_of("noalloc", n, len(wires), dt.__name__))
    sv = sv_class(ops_module, dt)(n)
    sv.updateData(rand_state(rng, n, dt))
    h = rand_hermitian(rng, len(wires))
    rc, ref = _expval("plgb_meas_expval_matrix", sv, h, wires)
    assert rc == 0
    for call in range(2):
        rc, got = _expval("plgb_meas_expval_matrix_noalloc", sv, h, wires)
        assert rc == 0, _capi.lib().plgb_last_error().decode()
        # an expectation value's error scales with ||h||
        assert_scalar(got, ref, dt, mag=float(np.linalg.norm(h, 2)), what=f"no-alloc call {call}")


def test_noalloc_two_state_vectors_in_a_row(ops_module):
    # the shared array holds nothing between calls: alternate two registers
    rng = np.random.default_rng(seed_of("noalloc-two"))
    a = sv_class(ops_module, np.complex128)(10)
    b = sv_class(ops_module, np.complex64)(11)
    a.updateData(rand_state(rng, 10, np.complex128))
    b.updateData(rand_state(rng, 11, np.complex64))
    ha, hb = rand_hermitian(rng, 2), rand_hermitian(rng, 3)
    ra = _expval("plgb_meas_expval_matrix", a, ha, [1, 6])[1]
    rb = _expval("plgb_meas_expval_matrix", b, hb, [0, 4, 10])[1]
    for _ in range(2):
        assert_scalar(_expval("plgb_meas_expval_matrix_noalloc", a, ha, [1, 6])[1], ra, np.complex128,
                      mag=float(np.linalg.norm(ha, 2)), what="a")
        assert_scalar(_expval("plgb_meas_expval_matrix_noalloc", b, hb, [0, 4, 10])[1], rb, np.complex64,
                      mag=float(np.linalg.norm(hb, 2)), what="b")


def test_noalloc_rejects_more_than_five_wires(ops_module):
    sv = sv_class(ops_module, np.complex128)(8)
    h = rand_hermitian(np.random.default_rng(0), 6)
    rc, _ = _expval("plgb_meas_expval_matrix_noalloc", sv, h, [0, 1, 2, 3, 4, 5])
    assert rc != 0
    assert "at most 5 wires" in _capi.lib().plgb_last_error().decode()
    # the allocating entry point still takes six wires
    rc, _ = _expval("plgb_meas_expval_matrix", sv, h, [0, 1, 2, 3, 4, 5])
    assert rc == 0


def _allocations():
    n = C.c_uint64(0)
    assert _capi.lib().plgb_device_allocations(C.byref(n)) == 0
    return n.value


def test_noalloc_makes_no_device_allocation(ops_module):
    # the property the entry point is named for: across two calls the
    # library requests no device memory (the allocating entry point does,
    # the first time it stages a matrix of that size)
    rng = np.random.default_rng(seed_of("noalloc-count"))
    sv = sv_class(ops_module, np.complex128)(12)
    sv.updateData(rand_state(rng, 12, np.complex128))
    h = rand_hermitian(rng, 5)
    before = _allocations()
    for _ in range(2):
        rc, _ = _expval("plgb_meas_expval_matrix_noalloc", sv, h, [0, 3, 5, 7, 11])
        assert rc == 0
    assert _allocations() == before


def test_noalloc_rejects_queued_gates(ops_module):
    # a lazy handle (17 qubits and up) queues gate calls; running the queue
    # compiles a fused program and allocates, so the call refuses until the
    # queue has run, then matches the allocating entry point
    n = 17
    sv = sv_class(ops_module, np.complex128)(n)
    for q in range(n):
        sv.RX([q], False, [0.1 + 0.05 * q])
        sv.CNOT([q, (q + 1) % n], False, [])
    h = rand_hermitian(np.random.default_rng(1), 2)
    before = _allocations()
    rc, _ = _expval("plgb_meas_expval_matrix_noalloc", sv, h, [2, 9])
    assert rc != 0
    assert "queued" in _capi.lib().plgb_last_error().decode()
    assert _allocations() == before
    assert _capi.lib().plgb_sv_synchronize(sv._h) == 0  # runs the queue
    ref = _expval("plgb_meas_expval_matrix", sv, h, [2, 9])[1]
    mark = _allocations()
    rc, got = _expval("plgb_meas_expval_matrix_noalloc", sv, h, [2, 9])
    assert rc == 0
    assert_scalar(got, ref, np.complex128, mag=float(np.linalg.norm(h, 2)), what="after the queue ran")
    assert _allocations() == mark
