"""torch.autograd path (lightning_gb300.torch_adjoint): the adjoint backward
against central finite differences (h = 1e-4, tolerance 1e-7 absolute on
O(1) gradients: truncation ~h^2 |f'''|/6) and against the oracle's adjoint
Jacobian (1e-12 relative for complex128, 1e-5 for complex64), checkpointed
and stored-state modes, shared parameters, and the in-place C entry point."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from helpers import assert_close  # noqa: E402
from lightning_gb300.torch_adjoint import ParamCircuit, ParamOp, config3_circuit, expval, jacobian  # noqa: E402
from lightning_gb300.workloads import PauliSum  # noqa: E402

pytestmark = pytest.mark.gpu


def fd_grad(circ, theta, idx, h=1e-4):
    out = []
    for k in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        ep = expval(torch.tensor(tp), circ).item()
        em = expval(torch.tensor(tm), circ).item()
        out.append((ep - em) / (2 * h))
    return np.array(out)


def test_grad_vs_central_differences():
    circ, theta = config3_circuit(n=8, layers=3, nterms=20)
    t = torch.tensor(theta, requires_grad=True)
    e = expval(t, circ)
    e.backward()
    g = t.grad.numpy()
    rng = np.random.default_rng(7)
    idx = sorted(rng.choice(theta.size, size=32, replace=False))
    fd = fd_grad(circ, theta, idx)
    assert np.max(np.abs(g[idx] - fd)) < 1e-7, np.max(np.abs(g[idx] - fd))


@pytest.mark.parametrize("precision,tol", [(128, 1e-12), (64, 1e-5)])
def test_grad_vs_oracle_adjoint(oracle, precision, tol):
    from oracle.pyoracle import pauli_sum_spec

    circ, theta = config3_circuit(n=10, layers=2, nterms=30, precision=precision)
    t = torch.tensor(theta, requires_grad=True)
    expval(t, circ).backward()
    dt = np.complex128 if precision == 128 else np.complex64
    st = np.zeros(1 << 10, dt)
    st[0] = 1
    ops = [dict(name=op.name, wires=op.wires, params=[theta[op.param]] if op.param is not None else [])
           for op in circ.ops]
    ref = oracle.sv(10, dt)
    ref.set_state(st)
    jac = ref.adjoint(ops, [pauli_sum_spec(circ.hamiltonian.terms())], list(range(theta.size)), apply_ops=True)[0]
    assert_close(t.grad.numpy(), jac, dt, what="autograd vs oracle adjoint")


def test_checkpoint_equals_stored_state():
    circ, theta = config3_circuit(n=9, layers=2, nterms=10, checkpoint=True)
    a = torch.tensor(theta, requires_grad=True)
    expval(a, circ).backward()
    circ2, _ = config3_circuit(n=9, layers=2, nterms=10, checkpoint=False)
    b = torch.tensor(theta, requires_grad=True)
    e2 = expval(b, circ2)
    e2.backward(retain_graph=True)
    gb = b.grad.clone()
    b.grad = None
    e2.backward()  # stored state survives: the copy-based sweep does not consume it
    assert np.array_equal(a.grad.numpy(), gb.numpy())
    assert np.array_equal(gb.numpy(), b.grad.numpy())


def test_shared_parameters_and_fixed_gates():
    ham = PauliSum([0.7, -1.3], ["ZZ", "X"], [[0, 1], [2]])
    ops = [ParamOp("RX", [0], 0), ParamOp("RY", [1], 1), ParamOp("CNOT", [0, 1]), ParamOp("RZ", [1], 0),
           ParamOp("RY", [2], 1), ParamOp("RX", [2], None, value=0.3), ParamOp("CNOT", [1, 2]),
           ParamOp("RZ", [2], 2, inverse=True)]
    circ = ParamCircuit(3, ops, ham, tile_bits=0)
    theta = np.array([0.4, -1.1, 2.3])
    t = torch.tensor(theta, requires_grad=True)
    (2.0 * expval(t, circ)).backward()
    fd = 2.0 * fd_grad(circ, theta, [0, 1, 2])
    assert np.max(np.abs(t.grad.numpy() - fd)) < 1e-7


def test_inplace_jacobian_matches_copying_entry():
    circ, theta = config3_circuit(n=11, layers=2, nterms=15)
    a = jacobian(circ, theta, in_place=True)
    sv, S = circ.run(theta)
    b = jacobian(circ, theta, sv=sv, S=S, in_place=False)
    assert np.array_equal(a, b)


def test_double_float_sweep_matches_fp64(ops_module):
    # the fused adjoint sweep runs in FP64 by default; the opt-in
    # double-float sweep must agree within the complex128 tolerance
    circ, theta = config3_circuit(n=12, layers=3, nterms=25)
    b = jacobian(circ, theta, in_place=True)
    prev = ops_module.set_c128_fp64_passes(False)
    try:
        a = jacobian(circ, theta, in_place=True)
    finally:
        ops_module.set_c128_fp64_passes(prev)
    assert_close(a, b, np.complex128, what="double-float vs FP64 sweep")
    assert not np.array_equal(a, b)
