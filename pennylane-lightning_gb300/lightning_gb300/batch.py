"""Batched execution of many independent circuits on one GB300.

lightning.qubit runs one circuit at a time and crosses from Python into C++
once per gate (pennylane_lightning/lightning_qubit/_state_vector.py:220-299).
The batch engine takes many circuits at once, in packed arrays, and runs them
together: every circuit is compiled into fused tile passes on the host's
cores, pass k of all circuits is ONE persistent kernel launch over all their
tiles, and all Pauli-sum expectation values are ONE batched reduction.

A circuit's results do not depend on the rest of the batch: they are
bit-identical whether it runs alone or among thousands of others.

    packed = pack(circuits)            # or workloads.config2_packed(...)
    engine = BatchEngine(precision=128)
    values = engine.run(packed)        # one value per observable
"""
from __future__ import annotations

import ctypes as C
import json
from dataclasses import dataclass

import numpy as np

from ._capi import VP, call, lib

MAX_WIRES_PER_OP = 4
MAX_PARAMS_PER_OP = 3


def gate_codes() -> dict[str, int]:
    """Name -> code table of the packed format (plgb_gate_name)."""
    out, k = {}, 0
    while True:
        name = lib().plgb_gate_name(k)
        if not name:
            return out
        out[name.decode()] = k
        k += 1


_CODES: dict[str, int] | None = None
_NPAR = None
_NO_PARAM = {"Identity", "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "SX", "T", "CNOT", "CY", "CZ", "SWAP",
             "Toffoli", "CSWAP"}


def code_of(name: str) -> int:
    global _CODES
    if _CODES is None:
        _CODES = gate_codes()
    if name not in _CODES:
        raise ValueError(f"gate {name!r} is not supported by the batch engine (named gates only)")
    return _CODES[name]


@dataclass
class PackedBatch:
    """Circuits in flat arrays (the layout plgb_batch_run reads)."""

    num_qubits: np.ndarray    # int32 [C]
    op_offsets: np.ndarray    # int64 [C + 1]
    op_codes: np.ndarray      # int32 [M]
    op_wires: np.ndarray      # int32 [M, 4], -1 = unused
    op_params: np.ndarray     # float64 [M, 3]
    op_inverse: np.ndarray    # uint8 [M]
    obs_offsets: np.ndarray   # int64 [C + 1]
    term_offsets: np.ndarray  # int64 [K + 1]
    term_coeffs: np.ndarray   # float64 [T]
    term_x: np.ndarray        # uint64 [T], bit w = X on wire w
    term_y: np.ndarray
    term_z: np.ndarray

    @property
    def num_circuits(self) -> int:
        return int(self.num_qubits.shape[0])

    @property
    def num_observables(self) -> int:
        return int(self.term_offsets.shape[0] - 1)

    def observables_of(self, values: np.ndarray) -> list[np.ndarray]:
        """Split a run's output into one array per circuit."""
        return [values[self.obs_offsets[c]:self.obs_offsets[c + 1]] for c in range(self.num_circuits)]

    def select(self, idx) -> "PackedBatch":
        """A batch of the circuits idx (in that order)."""
        parts = []
        for c in idx:
            o0, o1 = int(self.op_offsets[c]), int(self.op_offsets[c + 1])
            b0, b1 = int(self.obs_offsets[c]), int(self.obs_offsets[c + 1])
            t0, t1 = int(self.term_offsets[b0]), int(self.term_offsets[b1])
            parts.append((c, o0, o1, b0, b1, t0, t1))
        op_sel = np.concatenate([np.arange(p[1], p[2]) for p in parts]) if parts else np.zeros(0, np.int64)
        t_sel = np.concatenate([np.arange(p[5], p[6]) for p in parts]) if parts else np.zeros(0, np.int64)
        op_off = np.concatenate([[0], np.cumsum([p[2] - p[1] for p in parts])]).astype(np.int64)
        obs_off = np.concatenate([[0], np.cumsum([p[4] - p[3] for p in parts])]).astype(np.int64)
        nterms = [int(self.term_offsets[b + 1] - self.term_offsets[b]) for p in parts for b in range(p[3], p[4])]
        term_off = np.concatenate([[0], np.cumsum(nterms)]).astype(np.int64)
        return PackedBatch(self.num_qubits[list(idx)].astype(np.int32), op_off,
                           self.op_codes[op_sel], self.op_wires[op_sel], self.op_params[op_sel],
                           self.op_inverse[op_sel], obs_off, term_off, self.term_coeffs[t_sel],
                           self.term_x[t_sel], self.term_y[t_sel], self.term_z[t_sel])


def pauli_masks(word: str, wires) -> tuple[int, int, int]:
    x = y = z = 0
    for c, w in zip(word, wires):
        b = 1 << int(w)
        if c == "X":
            x |= b
        elif c == "Y":
            y |= b
        elif c == "Z":
            z |= b
        elif c != "I":
            raise ValueError(f"unknown Pauli letter {c!r}")
    return x, y, z


def pack(circuits) -> PackedBatch:
    """Pack circuits given as objects with `n`, `ops` (name, wires, params,
    inverse) and `observables` (Pauli sums with coeffs, words, wires)."""
    nq, op_off, obs_off, term_off = [], [0], [0], [0]
    codes, wires, params, inv = [], [], [], []
    coeffs, xs, ys, zs = [], [], [], []
    for circ in circuits:
        nq.append(int(circ.n))
        for op in circ.ops:
            if getattr(op, "matrix", None) is not None:
                raise ValueError("the batch engine takes named gates only")
            if len(op.wires) > MAX_WIRES_PER_OP or len(op.params) > MAX_PARAMS_PER_OP:
                raise ValueError(f"{op.name}: at most 4 wires and 3 parameters per operation")
            codes.append(code_of(op.name))
            wires.append(list(op.wires) + [-1] * (MAX_WIRES_PER_OP - len(op.wires)))
            params.append(list(op.params) + [0.0] * (MAX_PARAMS_PER_OP - len(op.params)))
            inv.append(1 if getattr(op, "inverse", False) else 0)
        op_off.append(len(codes))
        for obs in circ.observables:
            for c, word, ws in zip(obs.coeffs, obs.words, obs.wires):
                x, y, z = pauli_masks(word, ws)
                coeffs.append(float(c))
                xs.append(x)
                ys.append(y)
                zs.append(z)
            term_off.append(len(coeffs))
        obs_off.append(len(term_off) - 1)
    return PackedBatch(
        np.asarray(nq, np.int32), np.asarray(op_off, np.int64), np.asarray(codes, np.int32).reshape(-1),
        np.asarray(wires, np.int32).reshape(-1, MAX_WIRES_PER_OP),
        np.asarray(params, np.float64).reshape(-1, MAX_PARAMS_PER_OP), np.asarray(inv, np.uint8).reshape(-1),
        np.asarray(obs_off, np.int64), np.asarray(term_off, np.int64), np.asarray(coeffs, np.float64),
        np.asarray(xs, np.uint64), np.asarray(ys, np.uint64), np.asarray(zs, np.uint64))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class BatchEngine:
    """Runs PackedBatch objects; keeps its device arenas and tuned tile sizes
    between runs.  precision 64 (complex64) or 128 (complex128); tile_bits 0
    = autotuned per register size; wave_bytes 0 = 8 GiB of registers per
    wave; threads 0 = every host core for compilation."""

    def __init__(self, precision: int = 128, tile_bits: int = 0, wave_bytes: int = 0, threads: int = 0):
        self.precision = int(precision)
        self._h = VP()
        call("plgb_batch_create", self.precision, C.byref(self._h))
        call("plgb_batch_configure", self._h, int(tile_bits), int(wave_bytes), int(threads))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().plgb_batch_destroy(h)
            self._h = None

    def run(self, packed: PackedBatch) -> np.ndarray:
        p = packed
        arrays = [np.ascontiguousarray(a) for a in (
            p.num_qubits.astype(np.int32, copy=False), p.op_offsets.astype(np.int64, copy=False),
            p.op_codes.astype(np.int32, copy=False), p.op_wires.astype(np.int32, copy=False),
            p.op_params.astype(np.float64, copy=False), p.op_inverse.astype(np.uint8, copy=False),
            p.obs_offsets.astype(np.int64, copy=False), p.term_offsets.astype(np.int64, copy=False),
            p.term_coeffs.astype(np.float64, copy=False), p.term_x.astype(np.uint64, copy=False),
            p.term_y.astype(np.uint64, copy=False), p.term_z.astype(np.uint64, copy=False))]
        out = np.zeros(max(p.num_observables, 1), np.float64)
        call("plgb_batch_run", self._h, p.num_circuits, *[_ptr(a) for a in arrays],
             out.ctypes.data_as(C.POINTER(C.c_double)))
        return out[:p.num_observables]

    def _arrays(self, p: PackedBatch):
        return [np.ascontiguousarray(a) for a in (
            p.num_qubits.astype(np.int32, copy=False), p.op_offsets.astype(np.int64, copy=False),
            p.op_codes.astype(np.int32, copy=False), p.op_wires.astype(np.int32, copy=False),
            p.op_params.astype(np.float64, copy=False), p.op_inverse.astype(np.uint8, copy=False),
            p.obs_offsets.astype(np.int64, copy=False), p.term_offsets.astype(np.int64, copy=False),
            p.term_coeffs.astype(np.float64, copy=False), p.term_x.astype(np.uint64, copy=False),
            p.term_y.astype(np.uint64, copy=False), p.term_z.astype(np.uint64, copy=False))]

    def parametric_gates(self, p: PackedBatch) -> np.ndarray:
        """Number of parametric gates of each circuit (its Jacobian width)."""
        global _NPAR
        if _NPAR is None:
            _NPAR = np.array([0 if name in _NO_PARAM else 1 for name in sorted(gate_codes(), key=gate_codes().get)])
        per_op = _NPAR[p.op_codes] if p.op_codes.size else np.zeros(0, np.int64)
        cs = np.concatenate([[0], np.cumsum(per_op)]).astype(np.int64)
        return cs[p.op_offsets[1:]] - cs[p.op_offsets[:-1]]

    def run_adjoint(self, packed: PackedBatch):
        """<O> per observable and, per circuit, the Jacobian (observables x
        parametric gates) by the in-place adjoint sweep."""
        p = packed
        arrays = self._arrays(p)
        npar = self.parametric_gates(p)
        nobs = np.diff(p.obs_offsets)
        widths = npar * nobs
        values = np.zeros(max(p.num_observables, 1), np.float64)
        jac = np.zeros(max(int(widths.sum()), 1), np.float64)
        call("plgb_batch_adjoint", self._h, p.num_circuits, *[_ptr(a) for a in arrays],
             values.ctypes.data_as(C.POINTER(C.c_double)), jac.ctypes.data_as(C.POINTER(C.c_double)))
        offs = np.concatenate([[0], np.cumsum(widths)])
        jacs = [jac[offs[c]:offs[c + 1]].reshape(int(nobs[c]), int(npar[c])) for c in range(p.num_circuits)]
        return values[:p.num_observables], jacs

    def done_ms(self) -> list:
        """When each circuit of the last run had its results, in ms from the
        start of the run."""
        return self.stats().get("done_ms", [])

    def stats(self) -> dict:
        n = 1 << 16
        while True:
            buf = C.create_string_buffer(n)
            rc = lib().plgb_batch_stats(self._h, buf, n)
            if rc == 0:
                return json.loads(buf.value.decode())
            if n > (1 << 26):
                call("plgb_batch_stats", self._h, buf, n)
            n *= 4
