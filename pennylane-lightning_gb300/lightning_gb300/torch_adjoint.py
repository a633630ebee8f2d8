"""Differentiable expectation values for PyTorch, with the adjoint method on
the GPU as the hand-written backward.

    circ = ParamCircuit(num_qubits, ops, hamiltonian)   # ops: ParamOp(name, wires, param=index or None)
    e = expval(theta, circ)                              # <psi(theta)| H |psi(theta)>, psi = U(theta)|0..0>
    e.backward()                                         # theta.grad by the adjoint sweep

Forward: the circuit runs as fused tile passes (StateVector.applyOperations)
and <H> is one grouped Pauli reduction.  Backward: the adjoint sweep of
pennylane_lightning/core/simulators/lightning_qubit/algorithms/
AdjointJacobianLQubit.hpp:225-491 (applyOperationAdj, applyGenerator,
innerProduct), run on the GPU by plgb_adjoint_jacobian*; the Jacobian row of
the one observable is contracted with the incoming gradient and summed over
the gates that share a parameter.

State checkpointing (checkpoint=True, the default): the forward pass keeps no
state; the backward pass recomputes the final state and consumes it in
place, so at most 1 + 1 registers are alive (the state and H|state>).  At 32
qubits complex128 (64 GiB per register) that is what fits on one GB300.  With
checkpoint=False the forward state is kept and the backward works on a copy
(no recompute, two more registers).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import lightning_gb300_ops as ops
from ._capi import VP, call
from .workloads import PauliSum


@dataclass
class ParamOp:
    name: str
    wires: list[int]
    param: int | None = None   # index into theta, or None for a fixed gate
    inverse: bool = False
    value: float | None = None  # parameter of a fixed parametric gate


@dataclass
class ParamCircuit:
    num_qubits: int
    ops: list[ParamOp]
    hamiltonian: PauliSum
    precision: int = 128
    tile_bits: int = 11
    checkpoint: bool = True
    _obs_cache: dict = field(default_factory=dict, repr=False)

    def ops_struct(self, theta: np.ndarray):
        names, params, wires, inv = [], [], [], []
        for op in self.ops:
            names.append(op.name)
            if op.param is not None:
                params.append([float(theta[op.param])])
            elif op.value is not None:
                params.append([float(op.value)])
            else:
                params.append([])
            wires.append(list(op.wires))
            inv.append(bool(op.inverse))
        OS = ops.OpsStructC128 if self.precision == 128 else ops.OpsStructC64
        return OS(names, params, wires, inv, [None] * len(names))

    def observable(self):
        if "H" not in self._obs_cache:
            s = "C128" if self.precision == 128 else "C64"
            NO = getattr(ops.observables, "NamedObs" + s)
            TP = getattr(ops.observables, "TensorProdObs" + s)
            HA = getattr(ops.observables, "Hamiltonian" + s)
            names = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ", "I": "Identity"}
            h = self.hamiltonian
            self._obs_cache["H"] = HA(list(h.coeffs), [TP([NO(names[c], [w]) for c, w in zip(word, ws)])
                                                       for word, ws in zip(h.words, h.wires)])
        return self._obs_cache["H"]

    def param_ops(self) -> list[ParamOp]:
        """The operations that carry a parameter, in order (the adjoint's
        trainable-parameter numbering)."""
        return [op for op in self.ops if op.param is not None or op.value is not None]

    def run(self, theta: np.ndarray):
        SV = ops.StateVectorC128 if self.precision == 128 else ops.StateVectorC64
        sv = SV(self.num_qubits)
        S = self.ops_struct(theta)
        sv.applyOperations(S, min(self.tile_bits, self.num_qubits) if self.tile_bits else 0)
        return sv, S


def _expval(circ: ParamCircuit, sv) -> float:
    M = ops.MeasurementsC128 if circ.precision == 128 else ops.MeasurementsC64
    return float(M(sv).expval(circ.observable()))


def jacobian(circ: ParamCircuit, theta: np.ndarray, sv=None, S=None, in_place: bool = True) -> np.ndarray:
    """d<H>/d(parameter of each parametric gate), in gate order.  With
    in_place the register (recomputed when not given) is consumed."""
    if sv is None:
        sv, S = circ.run(theta)
    pops = circ.param_ops()
    out = np.zeros(max(1, len(pops)), np.float64)
    tp = np.arange(len(pops), dtype=np.int64)
    arr = (VP * 1)(circ.observable()._h)
    tptr = tp.ctypes.data_as(C.POINTER(C.c_int64))
    optr = out.ctypes.data_as(C.POINTER(C.c_double))
    if in_place:
        call("plgb_adjoint_jacobian_inplace", sv._h, arr, 1, S._h, tptr, len(pops), optr)
    else:
        call("plgb_adjoint_jacobian", sv._h, arr, 1, S._h, tptr, len(pops), 0, optr)
    return out[:len(pops)]


class AdjointExpval(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta: torch.Tensor, circ: ParamCircuit):
        th = theta.detach().to("cpu", torch.float64).numpy()
        sv, S = circ.run(th)
        e = _expval(circ, sv)
        ctx.circ = circ
        ctx.theta = th
        if circ.checkpoint:
            del sv, S  # recomputed in backward
            ctx.state = None
        else:
            ctx.state = (sv, S)
        return torch.tensor(e, dtype=theta.dtype, device=theta.device)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        circ = ctx.circ
        if ctx.state is None:
            jac = jacobian(circ, ctx.theta, in_place=True)
        else:
            sv, S = ctx.state
            jac = jacobian(circ, ctx.theta, sv=sv, S=S, in_place=False)
        grad = np.zeros(ctx.theta.shape[0], np.float64)
        for k, op in enumerate(circ.param_ops()):
            if op.param is not None:
                grad[op.param] += jac[k]
        g = torch.as_tensor(grad, dtype=grad_out.dtype, device=grad_out.device) * grad_out
        return g, None


def expval(theta: torch.Tensor, circ: ParamCircuit) -> torch.Tensor:
    return AdjointExpval.apply(theta, circ)


def config3_circuit(n: int = 28, layers: int = 12, seed: int = 1003, nterms: int = 200, precision: int = 128,
                    checkpoint: bool = True, tile_bits: int = 11):
    """The strongly entangling benchmark circuit with one parameter per
    rotation; returns (circuit, initial theta)."""
    from .workloads import config3

    body, ham = config3(n, layers, seed, nterms)
    pops, theta = [], []
    for op in body:
        if op.params:
            pops.append(ParamOp(op.name, list(op.wires), param=len(theta)))
            theta.append(op.params[0])
        else:
            pops.append(ParamOp(op.name, list(op.wires)))
    return ParamCircuit(n, pops, ham, precision, tile_bits, checkpoint), np.asarray(theta, np.float64)
