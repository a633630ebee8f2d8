"""Python binding of the GB300 backend with the names of ``lightning_qubit_ops``.

Mirrors the module the reference builds from
pennylane_lightning/core/bindings/Bindings.hpp and
pennylane_lightning/core/simulators/lightning_qubit/bindings/LQubitBindings.hpp:
``StateVectorC64/C128`` (one method per gate name, plain and controlled
overloads), ``MeasurementsC64/C128``, the ``observables`` and ``algorithms``
namespaces, ``allocate_aligned_array``, ``compile_info``, ``runtime_info`` and
``backend_info``.  Every call goes through the C ABI of include/pl_gb300.h;
errors raise ``LightningException`` (a RuntimeError), as the reference's
``PL_ABORT`` does through nanobind.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import types
from typing import Sequence

import numpy as np

from ._capi import DP, I64P, IP, U8P, VP, LightningException, call, lib

__all__ = [
    "StateVectorC64", "StateVectorC128", "MeasurementsC64", "MeasurementsC128", "observables", "algorithms",
    "allocate_aligned_array", "compile_info", "runtime_info", "backend_info", "LightningException",
]

# Constant.hpp gate_names / controlled_gate_names
GATE_NAMES = (
    "Identity", "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "SX", "T", "PhaseShift", "RX", "RY", "RZ", "Rot",
    "CNOT", "CY", "CZ", "IsingXX", "IsingXY", "IsingYY", "IsingZZ", "SWAP", "ControlledPhaseShift", "CRX", "CRY",
    "CRZ", "CRot", "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus", "Toffoli", "CSWAP",
    "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus", "MultiRZ", "GlobalPhase", "PSWAP",
    "PCPhase",
)
CONTROLLED_GATE_NAMES = (
    "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "SX", "T", "PhaseShift", "RX", "RY", "RZ", "Rot", "SWAP",
    "IsingXX", "IsingXY", "IsingYY", "IsingZZ", "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus",
    "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus", "MultiRZ", "GlobalPhase", "PSWAP", "PCPhase",
)


# --------------------------------------------------------------------------- helpers
def _i64(xs) -> tuple[object, int]:
    xs = [int(x) for x in (xs if xs is not None else [])]
    arr = (C.c_int64 * max(1, len(xs)))(*xs)
    return arr, len(xs)


def _u8(xs) -> object:
    xs = [1 if bool(x) else 0 for x in (xs if xs is not None else [])]
    return (C.c_uint8 * max(1, len(xs)))(*xs)


def _f64(xs) -> tuple[object, int]:
    xs = [float(x) for x in (xs if xs is not None else [])]
    return (C.c_double * max(1, len(xs)))(*xs), len(xs)


def _cmat(m) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, dtype=np.complex128).reshape(-1))


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(DP)


def _text(fn, *args, size=4096) -> str:
    buf = C.create_string_buffer(size)
    call(fn, *args, buf, size)
    return buf.value.decode()


# --------------------------------------------------------------------------- module functions
def set_tile_variant(precision: int, occ: bool) -> bool:
    """Register-tile kernel variant for complex64 (64) or complex128 (128):
    occ=True caps registers at 128 per thread (more resident warps);
    returns the previous setting."""
    rc = lib().plgb_set_tile_variant(int(precision), 1 if occ else 0)
    if rc < 0:
        raise LightningException("precision must be 64 or 128")
    return bool(rc)


def set_lazy_fusion(on: bool) -> bool:
    """Default for new state vectors: per-gate calls are queued and run as
    fused tile passes by the next call that reads or rewrites the state (on,
    the default) or applied one at a time (off).  Returns the previous
    default."""
    return bool(lib().plgb_set_lazy_fusion(1 if on else 0))


def set_lazy_min_qubits(q: int) -> int:
    """Smallest register (in qubits) whose per-gate calls are queued for
    lazy fusion; smaller ones apply each gate at its call.  Returns the
    previous value."""
    if int(q) < 1:
        raise ValueError("min_qubits must be >= 1")
    return int(lib().plgb_set_lazy_min_qubits(int(q)))


def set_c128_fp64_passes(on: bool) -> bool:
    """Fused complex128 passes (and batched passes and the fused adjoint
    sweep) in FP64 (True, the default) or, opted into, double-float
    arithmetic on the FP32 pipe (False: ~48 significant bits, FP32 exponent
    range); returns the previous setting."""
    return bool(lib().plgb_set_c128_fp64_passes(1 if on else 0))


def set_tc_dense(on: bool) -> bool:
    """Dense complex64 six-wire gates on the tensor cores (True, the
    default) or the CUDA cores; returns the previous setting."""
    return bool(lib().plgb_set_tc_dense(1 if on else 0))


def backend_info() -> dict:
    """LQubitBindings.hpp:464-475."""
    return json.loads(_text("plgb_backend_info"))


def runtime_info() -> dict:
    """Bindings.hpp:364-367 (CPU flags there; CUDA device details here)."""
    return json.loads(_text("plgb_runtime_info"))


def compile_info() -> dict:
    """Bindings.hpp:284-362."""
    info = runtime_info()
    return {"cpu.arch": os.uname().machine, "compiler.name": "nvcc", "compiler.version": info.get("cuda_compiled"),
            "AVX2": False, "AVX512F": False, "GPU.arch": info.get("compiled_for")}


def kernel_launches() -> int:
    """Kernels launched by the backend library so far in this process."""
    v = C.c_uint64()
    call("plgb_kernel_launches", C.byref(v))
    return int(v.value)


def allocate_aligned_array(size: int, dtype, zero_init: bool = False) -> np.ndarray:
    """Bindings.hpp:422-456: numpy array of `size` entries (64-byte aligned)."""
    dtype = np.dtype(dtype)
    raw = np.empty(size * dtype.itemsize + 64, dtype=np.uint8)
    off = (-raw.ctypes.data) % 64
    arr = raw[off: off + size * dtype.itemsize].view(dtype)
    if zero_init:
        arr[:] = 0
    return arr


# --------------------------------------------------------------------------- state vector
class _StateVectorBase:
    _precision = 128
    _dtype = np.complex128

    def __init__(self, num_qubits: int, *, _handle=None):
        self._h = VP()
        if _handle is not None:
            self._h = _handle
        else:
            call("plgb_sv_create", int(num_qubits), self._precision, C.byref(self._h))
        n = C.c_int()
        call("plgb_sv_num_qubits", self._h, C.byref(n))
        self._n = n.value

    @classmethod
    def from_device_pointer(cls, ptr: int, num_qubits: int):
        """Wrap caller-owned device memory (StateVectorLQubitRaw counterpart)."""
        h = VP()
        call("plgb_sv_create_raw", VP(ptr), int(num_qubits), cls._precision, C.byref(h))
        return cls(num_qubits, _handle=h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                lib().plgb_sv_destroy(h)
            except Exception:
                pass
            self._h = None

    # StateVectorBase -------------------------------------------------------
    def __len__(self) -> int:
        return 1 << self._n

    def size(self) -> int:
        return 1 << self._n

    @property
    def num_qubits(self) -> int:
        return self._n

    @property
    def dtype(self):
        return self._dtype

    def device_pointer(self) -> int:
        p = VP()
        call("plgb_sv_device_ptr", self._h, C.byref(p))
        return int(p.value or 0)

    def synchronize(self) -> None:
        call("plgb_sv_synchronize", self._h)

    def set_lazy(self, on: bool) -> None:
        """Queue per-gate calls and run them fused at the next state read
        (on) or apply each gate at once (off); the queue runs first."""
        call("plgb_sv_set_lazy", self._h, 1 if on else 0)

    def cuda_stream(self) -> int:
        """Address of the cudaStream_t this state vector's kernels run on."""
        p = VP()
        call("plgb_sv_stream", self._h, C.byref(p))
        return int(p.value or 0)

    def resetStateVector(self) -> None:
        call("plgb_sv_reset", self._h)

    def setBasisState(self, state=None, wires=None, async_=False, **kw):
        state = list(state) if state is not None else []
        wires = list(wires) if wires is not None else list(range(len(state)))
        b, nb = _i64(state)
        w, nw = _i64(wires)
        if nb != nw:
            raise LightningException("state and wires must have the same length")
        call("plgb_sv_set_basis_state", self._h, b, w, nw)

    def setStateVector(self, state, wires, async_=False, **kw):
        st = np.ascontiguousarray(np.asarray(state, dtype=self._dtype).reshape(-1))
        w, nw = _i64(wires)
        call("plgb_sv_set_state_vector", self._h, st.ctypes.data_as(VP), st.size, w, nw)

    def updateData(self, data) -> None:
        arr = np.ascontiguousarray(np.asarray(data, dtype=self._dtype))
        if arr.ndim != 1:
            raise ValueError("Array must be 1-dimensional")
        call("plgb_sv_update_data", self._h, arr.ctypes.data_as(VP), arr.size)

    def getState(self, state: np.ndarray) -> None:
        if not isinstance(state, np.ndarray) or state.dtype != self._dtype or not state.flags.c_contiguous:
            raise TypeError(f"getState expects a C-contiguous numpy array of dtype {np.dtype(self._dtype)}")
        if state.size < len(self):
            raise ValueError("Output array is too small")
        call("plgb_sv_get_state", self._h, state.ctypes.data_as(VP), state.size)

    def state(self) -> np.ndarray:
        out = np.empty(len(self), dtype=self._dtype)
        self.getState(out)
        return out

    # gates -----------------------------------------------------------------
    def _apply_named(self, name: str, wires, inverse: bool = False, params=()):
        w, nw = _i64(wires)
        p, npar = _f64(params)
        call("plgb_sv_apply_operation", self._h, name.encode(), w, nw, int(bool(inverse)), p, npar)

    def _apply_controlled(self, name, controlled_wires, controlled_values, wires, inverse=False, params=()):
        cw, ncw = _i64(controlled_wires)
        cv = _u8(controlled_values)
        if len(list(controlled_values)) != ncw:
            raise LightningException("`controlled_wires` must have the same size as `controlled_values`.")
        w, nw = _i64(wires)
        p, npar = _f64(params)
        call("plgb_sv_apply_controlled_operation", self._h, name.encode(), cw, cv, ncw, w, nw,
             int(bool(inverse)), p, npar)

    def applyOperation(self, name: str, wires, inverse: bool = False, params=(), controlled_wires=(),
                       controlled_values=(), matrix=None):
        """StateVectorLQubit.hpp:431-482: named if known, else the matrix."""
        if controlled_wires:
            if name in CONTROLLED_GATE_NAMES:
                return self._apply_controlled(name, controlled_wires, controlled_values, wires, inverse, params)
            return self.applyControlledMatrix(matrix, controlled_wires, controlled_values, wires, inverse)
        if name in GATE_NAMES:
            return self._apply_named(name, wires, inverse, params)
        if matrix is None:
            raise LightningException(f"Operation {name} is not supported and no matrix was given")
        return self.applyMatrix(matrix, wires, inverse)

    def applyOperations(self, ops, tile_bits: int = 0) -> int:
        """Apply an OpsStruct list (StateVectorBase::applyOperations).

        tile_bits = 0 runs one kernel per gate; tile_bits = t > 0 fuses the
        list into shared-memory tile passes of 2^t amplitudes (complex64
        registers of 22 qubits and more: dense blocks of up to six wires on
        the tensor cores while set_tc_dense is on).  Returns the number of
        kernel passes the call issued."""
        passes = C.c_int()
        call("plgb_sv_apply_operations", self._h, ops._h, int(tile_bits), C.byref(passes))
        return passes.value

    def applyOperationsBlocks(self, ops, block_wires: int) -> int:
        """Apply an OpsStruct list fused into dense blocks on at most
        block_wires (1..6) wires, one kernel per block (complex64 blocks of
        four to six wires on the tensor cores).  Returns the number of
        kernels the call issued."""
        blocks = C.c_int()
        call("plgb_sv_apply_operations_blocks", self._h, ops._h, int(block_wires), C.byref(blocks))
        return blocks.value

    def applyMatrix(self, matrix, wires, inverse: bool = False) -> None:
        m = _cmat(matrix)
        w, nw = _i64(wires)
        if m.size != 1 << (2 * nw):
            raise LightningException("The size of matrix does not match with the given number of wires")
        call("plgb_sv_apply_matrix", self._h, _dptr(m.view(np.float64)), w, nw, int(bool(inverse)))

    def applyControlledMatrix(self, matrix, controlled_wires, controlled_values, wires, inverse=False) -> None:
        m = _cmat(matrix)
        cw, ncw = _i64(controlled_wires)
        cv = _u8(controlled_values)
        w, nw = _i64(wires)
        if m.size != 1 << (2 * nw):
            raise LightningException("The size of matrix does not match with the given number of wires")
        call("plgb_sv_apply_controlled_matrix", self._h, _dptr(m.view(np.float64)), cw, cv, ncw, w, nw,
             int(bool(inverse)))

    def applySparseMatrix(self, row_map, col_idx, values, wires, inverse=False) -> None:
        self.applyControlledSparseMatrix(row_map, col_idx, values, [], [], wires, inverse)

    def applyControlledSparseMatrix(self, row_map, col_idx, values, controlled_wires, controlled_values, wires,
                                    inverse=False) -> None:
        if inverse:
            raise LightningException("Inverse not implemented for sparse ops.")
        ip = np.ascontiguousarray(np.asarray(row_map, dtype=np.int64))
        ix = np.ascontiguousarray(np.asarray(col_idx, dtype=np.int64))
        d = _cmat(values)
        cw, ncw = _i64(controlled_wires)
        cv = _u8(controlled_values)
        w, nw = _i64(wires)
        if ip.size - 1 != 1 << nw:
            raise LightningException("The size of matrix does not match with the given number of wires")
        call("plgb_sv_apply_sparse_matrix", self._h, ip.ctypes.data_as(I64P), ix.ctypes.data_as(I64P),
             _dptr(d.view(np.float64)), d.size, cw, cv, ncw, w, nw)

    def applyPauliRot(self, wires, inverse, params, word: str) -> None:
        w, nw = _i64(wires)
        call("plgb_sv_apply_pauli_rot", self._h, w, nw, int(bool(inverse)), float(params[0]), word.encode())

    def applyGenerator(self, name: str, wires, adj: bool = False, controlled_wires=(), controlled_values=()) -> float:
        w, nw = _i64(wires)
        cw, ncw = _i64(controlled_wires)
        cv = _u8(controlled_values)
        scale = C.c_double()
        call("plgb_sv_apply_generator", self._h, name.encode(), cw, cv, ncw, w, nw, int(bool(adj)),
             C.byref(scale))
        return scale.value

    def collapse(self, wire: int, branch: bool) -> None:
        call("plgb_sv_collapse", self._h, int(wire), int(bool(branch)))

    def normalize(self) -> None:
        call("plgb_sv_normalize", self._h)

    def kernel_map(self) -> dict:
        """LQubitBindings.hpp:209-228 svKernelMap: every op runs on the GB300 kernels."""
        return {name: "GB300" for name in GATE_NAMES}


def _gate_method(name: str):
    def method(self, *args, **kwargs):
        # Plain overload (wires, inverse, params) vs controlled overload
        # (controlled_wires, controlled_values, wires, inverse=False, params=[]),
        # resolved as nanobind does: the plain form needs a bool second argument.
        if "controlled_wires" in kwargs or "controlled_values" in kwargs:
            return self._apply_controlled(name, kwargs.pop("controlled_wires"), kwargs.pop("controlled_values"),
                                          *args, **kwargs)
        plain = len(args) + len(kwargs) <= 3 and (
            len(args) < 2 or isinstance(args[1], (bool, np.bool_, int)) and not isinstance(args[1], (list, tuple)))
        if plain:
            return self._apply_named(name, *args, **kwargs)
        if name not in CONTROLLED_GATE_NAMES:
            raise LightningException(f"Controlled gate {name} is not supported")
        return self._apply_controlled(name, *args, **kwargs)

    method.__name__ = name
    method.__doc__ = f"Apply the {name} gate (plain or controlled overload)."
    return method


for _g in GATE_NAMES:
    setattr(_StateVectorBase, _g, _gate_method(_g))


class StateVectorC128(_StateVectorBase):
    _precision = 128
    _dtype = np.complex128


class StateVectorC64(_StateVectorBase):
    _precision = 64
    _dtype = np.complex64


# --------------------------------------------------------------------------- observables
class _ObservableBase:
    _precision = 128

    def __init__(self, handle):
        self._h = handle

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                lib().plgb_obs_destroy(h)
            except Exception:
                pass
            self._h = None

    def get_wires(self) -> list[int]:
        n = C.c_int()
        call("plgb_obs_wires", self._h, None, 0, C.byref(n))
        buf = (C.c_int64 * max(1, n.value))()
        call("plgb_obs_wires", self._h, buf, n.value, C.byref(n))
        return [int(x) for x in buf[: n.value]]

    def __repr__(self) -> str:
        return _text("plgb_obs_repr", self._h)

    def __eq__(self, other) -> bool:
        return type(self) is type(other) and self._key() == other._key()

    def __hash__(self):
        return id(self)

    def _key(self):
        return repr(self)


def _obs_classes(precision: int):
    suffix = "C64" if precision == 64 else "C128"

    class NamedObs(_ObservableBase):
        _precision = precision

        def __init__(self, name: str, wires, params=None):
            h = VP()
            w, nw = _i64(wires)
            call("plgb_obs_named", name.encode(), w, nw, C.byref(h))
            super().__init__(h)
            self._name, self._wires = name, list(wires)

        def get_obs_name(self) -> str:
            return self._name

        def _key(self):
            return ("named", self._name, tuple(self._wires))

    class HermitianObs(_ObservableBase):
        _precision = precision

        def __init__(self, matrix, wires):
            m = _cmat(matrix)
            h = VP()
            w, nw = _i64(wires)
            call("plgb_obs_hermitian", _dptr(m.view(np.float64)), w, nw, C.byref(h))
            super().__init__(h)
            self._m, self._wires = m, list(wires)

        def get_matrix(self):
            return self._m.astype(np.complex64 if precision == 64 else np.complex128)

        def _key(self):
            return ("herm", self._m.tobytes(), tuple(self._wires))

    class TensorProdObs(_ObservableBase):
        _precision = precision

        def __init__(self, obs: Sequence[_ObservableBase]):
            self._obs = list(obs)
            arr = (VP * max(1, len(self._obs)))(*[o._h for o in self._obs])
            h = VP()
            call("plgb_obs_tensor_prod", arr, len(self._obs), C.byref(h))
            super().__init__(h)

        def get_ops(self):
            return list(self._obs)

        def _key(self):
            return ("prod", tuple(o._key() for o in self._obs))

    class Hamiltonian(_ObservableBase):
        _precision = precision

        def __init__(self, coeffs, obs: Sequence[_ObservableBase]):
            self._coeffs = [float(c) for c in np.asarray(coeffs, dtype=np.float64).reshape(-1)]
            self._obs = list(obs)
            if len(self._coeffs) != len(self._obs):
                raise LightningException("coeffs and observables must have the same length")
            c = (C.c_double * max(1, len(self._coeffs)))(*self._coeffs)
            arr = (VP * max(1, len(self._obs)))(*[o._h for o in self._obs])
            h = VP()
            call("plgb_obs_hamiltonian", c, arr, len(self._obs), C.byref(h))
            super().__init__(h)

        def get_coeffs(self):
            return np.asarray(self._coeffs, dtype=np.float32 if precision == 64 else np.float64)

        def get_ops(self):
            return list(self._obs)

        def _key(self):
            return ("ham", tuple(self._coeffs), tuple(o._key() for o in self._obs))

    class SparseHamiltonian(_ObservableBase):
        _precision = precision

        def __init__(self, data, indices, indptr, wires):
            d = _cmat(data)
            ix = np.ascontiguousarray(np.asarray(indices, dtype=np.int64))
            ip = np.ascontiguousarray(np.asarray(indptr, dtype=np.int64))
            w, nw = _i64(wires)
            h = VP()
            call("plgb_obs_sparse_hamiltonian", _dptr(d.view(np.float64)), ix.ctypes.data_as(I64P), ix.size,
                 ip.ctypes.data_as(I64P), ip.size, w, nw, C.byref(h))
            super().__init__(h)
            self._k = (d.tobytes(), ix.tobytes(), ip.tobytes(), tuple(wires))

        def _key(self):
            return ("sparse",) + self._k

    out = {}
    for cls, base in ((NamedObs, "NamedObs"), (HermitianObs, "HermitianObs"), (TensorProdObs, "TensorProdObs"),
                      (Hamiltonian, "Hamiltonian"), (SparseHamiltonian, "SparseHamiltonian")):
        cls.__name__ = cls.__qualname__ = base + suffix
        out[base + suffix] = cls
    out["Observable" + suffix] = _ObservableBase
    return out


observables = types.SimpleNamespace(**_obs_classes(64), **_obs_classes(128))


# --------------------------------------------------------------------------- measurements
class _MeasurementsBase:
    def __init__(self, sv: _StateVectorBase):
        self._sv = sv
        self._seed: int | None = None

    def set_random_seed(self, seed: int) -> None:
        self._seed = int(seed)

    def _next_seed(self) -> int:
        if self._seed is not None:
            return self._seed
        return int.from_bytes(os.urandom(4), "little")

    def probs(self, wires=None) -> np.ndarray:
        dt = np.float32 if self._sv._precision == 64 else np.float64
        if wires is None:
            out = np.empty(len(self._sv), dtype=np.float64)
            call("plgb_meas_probs", self._sv._h, None, -1, _dptr(out))
            return out.astype(dt)
        w, nw = _i64(wires)
        out = np.empty(1 << nw, dtype=np.float64)
        call("plgb_meas_probs", self._sv._h, w, nw, _dptr(out))
        return out.astype(dt)

    def generate_samples(self, wires_or_num, shots: int) -> np.ndarray:
        if isinstance(wires_or_num, (int, np.integer)):
            nw = int(wires_or_num)
            out = np.empty(shots * nw, dtype=np.int64)
            call("plgb_meas_generate_samples", self._sv._h, None, -1, int(shots), self._next_seed(),
                 out.ctypes.data_as(I64P))
            return out.reshape(shots, nw).astype(np.uint64)
        w, nw = _i64(wires_or_num)
        out = np.empty(max(1, shots * nw), dtype=np.int64)
        call("plgb_meas_generate_samples", self._sv._h, w, nw, int(shots), self._next_seed(),
             out.ctypes.data_as(I64P))
        return out[: shots * nw].reshape(shots, nw).astype(np.uint64)

    def generate_mcmc_samples(self, num_wires, kernelname, num_burnin, num_shots):
        """Metropolis-Hastings samples, shape (num_shots, num_wires), num_wires
        = the register's qubits (LQubitBindings.hpp:340-349)."""
        n = self._sv._n
        if int(num_wires) != n:
            raise LightningException(f"generate_mcmc_samples samples all {n} qubits (num_wires = {num_wires})")
        shots = int(num_shots)
        out = np.empty(max(1, shots * n), dtype=np.int64)
        call("plgb_meas_generate_mcmc_samples", self._sv._h, str(kernelname).encode(), int(num_burnin), shots,
             self._next_seed(), out.ctypes.data_as(I64P))
        return out[: shots * n].reshape(shots, n).astype(np.uint64)

    def expval(self, *args):
        r = C.c_double()
        if len(args) == 1:
            call("plgb_meas_expval_obs", self._sv._h, args[0]._h, C.byref(r))
        elif len(args) == 2 and isinstance(args[0], str):
            w, nw = _i64(args[1])
            call("plgb_meas_expval_named", self._sv._h, args[0].encode(), w, nw, C.byref(r))
        elif len(args) == 2:
            m = _cmat(args[0])
            w, nw = _i64(args[1])
            call("plgb_meas_expval_matrix", self._sv._h, _dptr(m.view(np.float64)), w, nw, C.byref(r))
        elif len(args) == 3:
            ip = np.ascontiguousarray(np.asarray(args[0], dtype=np.int64))
            ix = np.ascontiguousarray(np.asarray(args[1], dtype=np.int64))
            d = _cmat(args[2])
            call("plgb_meas_expval_sparse", self._sv._h, ip.ctypes.data_as(I64P), ip.size, ix.ctypes.data_as(I64P),
                 _dptr(d.view(np.float64)), d.size, C.byref(r))
        else:
            raise TypeError("expval(obs) | expval(name, wires) | expval(matrix, wires) | expval(row_map, col_idx, values)")
        return r.value

    def var(self, *args):
        r = C.c_double()
        if len(args) == 1:
            call("plgb_meas_var_obs", self._sv._h, args[0]._h, C.byref(r))
        elif len(args) == 2 and isinstance(args[0], str):
            w, nw = _i64(args[1])
            call("plgb_meas_var_named", self._sv._h, args[0].encode(), w, nw, C.byref(r))
        elif len(args) == 2:
            m = _cmat(args[0])
            w, nw = _i64(args[1])
            call("plgb_meas_var_matrix", self._sv._h, _dptr(m.view(np.float64)), w, nw, C.byref(r))
        elif len(args) == 3:
            ip = np.ascontiguousarray(np.asarray(args[0], dtype=np.int64))
            ix = np.ascontiguousarray(np.asarray(args[1], dtype=np.int64))
            d = _cmat(args[2])
            call("plgb_meas_var_sparse", self._sv._h, ip.ctypes.data_as(I64P), ip.size, ix.ctypes.data_as(I64P),
                 _dptr(d.view(np.float64)), d.size, C.byref(r))
        else:
            raise TypeError("var(obs) | var(name, wires) | var(matrix, wires) | var(row_map, col_idx, values)")
        return r.value


class MeasurementsC128(_MeasurementsBase):
    pass


class MeasurementsC64(_MeasurementsBase):
    pass


# --------------------------------------------------------------------------- algorithms
class _OpsStructBase:
    """OpsData (JacobianData.hpp:39-253)."""

    def __init__(self, names, params, wires, inverses, matrices, controlled_wires=None, controlled_values=None):
        n = len(names)
        controlled_wires = controlled_wires if controlled_wires is not None else [[] for _ in range(n)]
        controlled_values = controlled_values if controlled_values is not None else [[] for _ in range(n)]
        self.names, self.params, self.wires = list(names), [list(p) for p in params], [list(w) for w in wires]
        self.inverses = [bool(x) for x in inverses]
        self.matrices = [(_cmat(m) if m is not None and np.asarray(m).size else np.zeros(0, np.complex128))
                         for m in matrices]
        self.controlled_wires = [list(c) for c in controlled_wires]
        self.controlled_values = [list(c) for c in controlled_values]
        cnames = (C.c_char_p * max(1, n))(*[s.encode() for s in self.names])
        fp = [float(x) for p in self.params for x in p]
        params_a = (C.c_double * max(1, len(fp)))(*fp)
        nparams = (C.c_int * max(1, n))(*[len(p) for p in self.params])
        fw = [int(x) for w in self.wires for x in w]
        wires_a = (C.c_int64 * max(1, len(fw)))(*fw)
        nwires = (C.c_int * max(1, n))(*[len(w) for w in self.wires])
        inv = (C.c_uint8 * max(1, n))(*[int(x) for x in self.inverses])
        mflat = np.ascontiguousarray(np.concatenate(self.matrices) if any(m.size for m in self.matrices)
                                     else np.zeros(1, np.complex128))
        msz = (C.c_int64 * max(1, n))(*[m.size for m in self.matrices])
        fcw = [int(x) for c in self.controlled_wires for x in c]
        cw = (C.c_int64 * max(1, len(fcw)))(*fcw)
        ncw = (C.c_int * max(1, n))(*[len(c) for c in self.controlled_wires])
        fcv = [1 if bool(x) else 0 for c in self.controlled_values for x in c]
        cv = (C.c_uint8 * max(1, len(fcv)))(*fcv)
        self._h = VP()
        call("plgb_ops_create", n, cnames, params_a, nparams, wires_a, nwires, inv, _dptr(mflat.view(np.float64)),
             msz, cw, ncw, cv, C.byref(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                lib().plgb_ops_destroy(h)
            except Exception:
                pass
            self._h = None

    def fusion_plan(self, num_qubits: int, tile_bits: int) -> list:
        """The tile passes applyOperations(tile_bits) would run (no GPU needed)."""
        prec = 64 if isinstance(self, OpsStructC64) else 128
        buf = C.create_string_buffer(1 << 22)
        call("plgb_ops_fusion_plan", self._h, int(num_qubits), prec, int(tile_bits), buf, len(buf))
        return json.loads(buf.value.decode())

    def block_plan(self, num_qubits: int, block_wires: int, matrices: bool = False) -> list:
        """The dense blocks applyOperationsBlocks(block_wires) would run (no
        GPU needed): per block its kind, targets and (optionally) matrix."""
        prec = 64 if isinstance(self, OpsStructC64) else 128
        size = 1 << 22
        while True:
            buf = C.create_string_buffer(size)
            rc = lib().plgb_ops_block_plan(self._h, int(num_qubits), prec, int(block_wires), int(bool(matrices)),
                                           buf, len(buf))
            if rc == 0:
                return json.loads(buf.value.decode())
            msg = lib().plgb_last_error().decode()
            if msg != "buffer too small":
                raise LightningException(msg)
            size <<= 2

    def num_par_ops(self) -> int:
        k = C.c_int()
        call("plgb_ops_num_par_ops", self._h, C.byref(k))
        return k.value

    def __repr__(self) -> str:
        return f"Operations: [{', '.join(self.names)}]"


class OpsStructC128(_OpsStructBase):
    pass


class OpsStructC64(_OpsStructBase):
    pass


def create_ops_listC128(names, params, wires, inverses, matrices, controlled_wires, controlled_values):
    return OpsStructC128(names, params, wires, inverses, matrices, controlled_wires, controlled_values)


def create_ops_listC64(names, params, wires, inverses, matrices, controlled_wires, controlled_values):
    return OpsStructC64(names, params, wires, inverses, matrices, controlled_wires, controlled_values)


class _AdjointJacobianBase:
    """AdjointJacobianC*.__call__ (Bindings.hpp:704-729)."""

    def __call__(self, sv: _StateVectorBase, observables_list, ops: _OpsStructBase, trainable_params,
                 apply_operations: bool = False) -> np.ndarray:
        obs = list(observables_list)
        tp = [int(t) for t in trainable_params]
        out = np.zeros(max(1, len(obs) * len(tp)), dtype=np.float64)
        arr = (VP * max(1, len(obs)))(*[o._h for o in obs])
        t, ntp = _i64(tp)
        call("plgb_adjoint_jacobian", sv._h, arr, len(obs), ops._h, t, ntp, int(bool(apply_operations)), _dptr(out))
        dt = np.float32 if sv._precision == 64 else np.float64
        return out[: len(obs) * len(tp)].astype(dt)


class AdjointJacobianC128(_AdjointJacobianBase):
    pass


class AdjointJacobianC64(_AdjointJacobianBase):
    pass


class _VectorJacobianProductBase:
    """VectorJacobianProductC*.__call__ (LQubitBindings.hpp:412-457)."""

    def __call__(self, sv: _StateVectorBase, ops: _OpsStructBase, dy, trainable_params) -> np.ndarray:
        tp = [int(t) for t in trainable_params]
        d = np.ascontiguousarray(np.asarray(dy, dtype=np.complex128).reshape(-1))
        if d.size != len(sv):
            raise LightningException("the cotangent must have one entry per amplitude")
        out = np.zeros(2 * max(1, len(tp)), dtype=np.float64)
        t, ntp = _i64(tp)
        call("plgb_vjp", sv._h, ops._h, _dptr(d.view(np.float64)), t, ntp, _dptr(out))
        dt = np.complex64 if sv._precision == 64 else np.complex128
        return out[: 2 * len(tp)].view(np.complex128).astype(dt)


class VectorJacobianProductC128(_VectorJacobianProductBase):
    pass


class VectorJacobianProductC64(_VectorJacobianProductBase):
    pass


algorithms = types.SimpleNamespace(
    OpsStructC64=OpsStructC64, OpsStructC128=OpsStructC128, create_ops_listC64=create_ops_listC64,
    create_ops_listC128=create_ops_listC128, AdjointJacobianC64=AdjointJacobianC64,
    AdjointJacobianC128=AdjointJacobianC128, VectorJacobianProductC64=VectorJacobianProductC64,
    VectorJacobianProductC128=VectorJacobianProductC128,
)
