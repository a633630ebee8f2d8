"""Lazy fusion of per-gate calls: gate calls on a lazy state vector are
queued and run as fused tile passes by the next call that reads the state.
The results must equal the gates applied one at a time (within the
precision's tolerance), errors must surface at the gate call, and reads in
the middle of a circuit must see every gate queued before them."""
import numpy as np
import pytest

from helpers import DTYPES, assert_close, meas_class, rand_unitary, seed_of, sv_class

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def queue_small_registers(ops_module):
    # the queue normally starts at 17 qubits; these tests run it on small ones
    prev = ops_module.set_lazy_min_qubits(1)
    yield
    ops_module.set_lazy_min_qubits(prev)


def _circuit(rng, n, depth):
    ops = []
    for _ in range(depth):
        for q in range(n):
            ops.append(("RX", [q], [float(rng.uniform(0, 6.28))]))
            ops.append(("RZ", [q], [float(rng.uniform(0, 6.28))]))
        for q in range(0, n - 1, 2):
            ops.append(("CNOT", [q, q + 1], []))
        ops.append(("matrix", [int(rng.integers(0, n)), int(rng.integers(0, n))], rand_unitary(rng, 2)))
        ops.append(("CRY", [int(rng.integers(0, n)), int(rng.integers(0, n))], [float(rng.uniform(0, 6.28))]))
        ops.append(("IsingZZ", [0, n - 1], [0.37]))
        ops.append(("ctrl", [int(rng.integers(0, n)), int(rng.integers(0, n))], [float(rng.uniform(0, 6.28))]))
    return ops


def _apply(sv, ops):
    for name, w, p in ops:
        if len(w) == 2 and w[0] == w[1]:
            continue
        if name == "matrix":
            sv.applyMatrix(p, w, False)
        elif name == "ctrl":
            sv.RY([w[0]], [True], [w[1]], False, p)
        else:
            getattr(sv, name)(w, False, p)


@pytest.mark.parametrize("dt", DTYPES)
def test_lazy_equals_eager(ops_module, dt):
    rng = np.random.default_rng(seed_of("lazy", dt.__name__))
    n = 12
    ops = _circuit(rng, n, 6)
    eager = sv_class(ops_module, dt)(n)
    eager.set_lazy(False)
    lazy = sv_class(ops_module, dt)(n)
    lazy.set_lazy(True)
    _apply(eager, ops)
    _apply(lazy, ops)
    a = np.zeros(1 << n, dtype=dt)
    b = np.zeros(1 << n, dtype=dt)
    eager.getState(a)
    lazy.getState(b)
    assert_close(b, a, dt, what="lazy state")
    # a read in the middle sees every gate queued before it
    half = len(ops) // 2
    e2 = sv_class(ops_module, dt)(n)
    e2.set_lazy(False)
    l2 = sv_class(ops_module, dt)(n)
    l2.set_lazy(True)
    _apply(e2, ops[:half])
    _apply(l2, ops[:half])
    assert_close(meas_class(ops_module, dt)(l2).probs(), meas_class(ops_module, dt)(e2).probs(), dt,
                 what="probs mid-circuit")
    _apply(e2, ops[half:])
    _apply(l2, ops[half:])
    e2.getState(a)
    l2.getState(b)
    assert_close(b, a, dt, what="state after mid-circuit read")


def test_lazy_errors_surface_at_the_call(ops_module):
    from lightning_gb300.lightning_gb300_ops import LightningException

    sv = sv_class(ops_module, np.complex128)(10)
    sv.set_lazy(True)
    sv.RX([3], False, [0.2])
    with pytest.raises(LightningException):
        sv.RX([10], False, [0.2])  # wire out of range
    with pytest.raises(LightningException):
        sv.CNOT([2, 2], False, [])  # repeated wire
    # the valid gate before the errors still applies
    ref = sv_class(ops_module, np.complex128)(10)
    ref.set_lazy(False)
    ref.RX([3], False, [0.2])
    a = np.zeros(1 << 10, dtype=np.complex128)
    b = np.zeros(1 << 10, dtype=np.complex128)
    sv.getState(a)
    ref.getState(b)
    assert_close(a, b, np.complex128)


def test_small_registers_apply_at_the_call(ops_module):
    # below the threshold a gate call launches its kernel at once; at or
    # above it the call only queues
    ops_module.set_lazy_min_qubits(17)
    small = sv_class(ops_module, np.complex128)(12)
    small.set_lazy(True)
    k0 = ops_module.kernel_launches()
    small.RX([3], False, [0.2])
    assert ops_module.kernel_launches() > k0
    big = sv_class(ops_module, np.complex128)(17)
    big.set_lazy(True)
    k1 = ops_module.kernel_launches()
    big.RX([3], False, [0.2])
    big.RY([4], False, [0.3])
    assert ops_module.kernel_launches() == k1
    big.synchronize()  # runs the queue
    assert ops_module.kernel_launches() > k1
    ref = sv_class(ops_module, np.complex128)(17)
    ref.set_lazy(False)
    ref.RX([3], False, [0.2])
    ref.RY([4], False, [0.3])
    a = np.zeros(1 << 17, dtype=np.complex128)
    b = np.zeros(1 << 17, dtype=np.complex128)
    big.getState(a)
    ref.getState(b)
    assert_close(a, b, np.complex128)
    with pytest.raises(ValueError):
        ops_module.set_lazy_min_qubits(0)
