"""ctypes driver for the CPU oracles (test infrastructure only).

``Oracle("orc")`` loads this repository's LM restatement (``liboracle.so``);
``Oracle("ref")`` loads the shim over the reference's own C++ headers
(``_ref/libplref.so``, present only where the reference checkout was
available to build it).  Both expose the C API of ``oracle_api.h``; this
module gives them one Python face so a test can drive either.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

_I64P = C.POINTER(C.c_int64)
_U8P = C.POINTER(C.c_uint8)
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)


def lib_path(kind: str) -> Path:
    return HERE / "liboracle.so" if kind == "orc" else HERE / "_ref" / "libplref.so"


def available(kind: str) -> bool:
    return lib_path(kind).exists()


_LIBS: dict[str, C.CDLL] = {}


def _load(kind: str) -> C.CDLL:
    if kind in _LIBS:
        return _LIBS[kind]
    path = lib_path(kind)
    if not path.exists():
        if kind == "orc":
            from . import build_oracle  # type: ignore

            build_oracle.build_restatement()
        else:
            raise FileNotFoundError(f"{path} is not built")
    lib = C.CDLL(str(path))
    p = kind + "_"
    sig = {
        "last_error": (C.c_char_p, []),
        "sv_new": (C.c_void_p, [C.c_int, C.c_int]),
        "sv_free": (None, [C.c_void_p]),
        "sv_set_state": (C.c_int, [C.c_void_p, C.c_void_p]),
        "sv_get_state": (C.c_int, [C.c_void_p, C.c_void_p]),
        "sv_apply": (C.c_int, [C.c_void_p, C.c_char_p, _I64P, _U8P, C.c_int, _I64P, C.c_int, C.c_int, _DP, C.c_int]),
        "sv_apply_matrix": (C.c_int, [C.c_void_p, _DP, _I64P, _U8P, C.c_int, _I64P, C.c_int, C.c_int]),
        "sv_apply_sparse": (C.c_int, [C.c_void_p, _I64P, _I64P, _DP, C.c_int64, _I64P, _U8P, C.c_int, _I64P, C.c_int]),
        "sv_apply_pauli_rot": (C.c_int, [C.c_void_p, _I64P, C.c_int, C.c_int, C.c_double, C.c_char_p]),
        "sv_apply_generator": (C.c_int, [C.c_void_p, C.c_char_p, _I64P, _U8P, C.c_int, _I64P, C.c_int, C.c_int, _DP]),
        "sv_collapse": (C.c_int, [C.c_void_p, C.c_int64, C.c_int]),
        "sv_normalize": (C.c_int, [C.c_void_p]),
        "sv_set_basis_state": (C.c_int, [C.c_void_p, _I64P, _I64P, C.c_int]),
        "probs": (C.c_int, [C.c_void_p, _I64P, C.c_int, _DP]),
        "expval_named": (C.c_int, [C.c_void_p, C.c_char_p, _I64P, C.c_int, _DP]),
        "expval_matrix": (C.c_int, [C.c_void_p, _DP, _I64P, C.c_int, _DP]),
        "var_named": (C.c_int, [C.c_void_p, C.c_char_p, _I64P, C.c_int, _DP]),
        "var_matrix": (C.c_int, [C.c_void_p, _DP, _I64P, C.c_int, _DP]),
        "expval_sparse": (C.c_int, [C.c_void_p, _I64P, C.c_int64, _I64P, _DP, C.c_int64, _DP]),
        "expval_obs": (C.c_int, [C.c_void_p, C.c_char_p, _DP, _I64P, _DP]),
        "var_obs": (C.c_int, [C.c_void_p, C.c_char_p, _DP, _I64P, _DP]),
        "samples": (C.c_int, [C.c_void_p, _I64P, C.c_int, C.c_int64, C.c_uint64, _I64P]),
        "mcmc_samples": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64, C.c_int64, C.c_uint64, _I64P]),
        "adjoint": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_char_p), _DP, _IP, _I64P, _IP, _U8P, _DP, _I64P,
                              _I64P, _IP, _U8P, C.c_int, C.POINTER(C.c_char_p), _DP, _I64P, _I64P, C.c_int,
                              C.c_int, _DP]),
        "vjp": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_char_p), _DP, _IP, _I64P, _IP, _U8P, _DP, _I64P,
                          _I64P, _IP, _U8P, _DP, _I64P, C.c_int, C.c_int, _DP]),
        "num_threads": (C.c_int, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, p + name)
        fn.restype = res
        fn.argtypes = args
    _LIBS[kind] = lib
    return lib


def _i64(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(list(x) if not isinstance(x, np.ndarray) else x, dtype=np.int64).reshape(-1))


def _u8(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(list(x), dtype=np.uint8).reshape(-1))


def _f64(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1))


def _c128(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.complex128).reshape(-1))


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


class ObsData:
    """Builds an observable spec string plus its complex/int side arrays."""

    def __init__(self):
        self.cdata: list[np.ndarray] = []
        self.ncd = 0
        self.idata: list[np.ndarray] = []
        self.nid = 0

    def add_matrix(self, m) -> int:
        m = _c128(m)
        off = self.ncd
        self.cdata.append(m)
        self.ncd += m.size
        return off

    def add_ints(self, v) -> int:
        v = _i64(v)
        off = self.nid
        self.idata.append(v)
        self.nid += v.size
        return off

    def arrays(self):
        cd = np.concatenate(self.cdata) if self.cdata else np.zeros(1, np.complex128)
        idd = np.concatenate(self.idata) if self.idata else np.zeros(1, np.int64)
        return np.ascontiguousarray(cd.view(np.float64)), np.ascontiguousarray(idd)


def pauli_sum_spec(terms, od: ObsData | None = None) -> str:
    """terms: list of (coeff, word, wires) -> 'ham' spec of TensorProd(NamedObs)."""
    names = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ", "I": "Identity", "H": "Hadamard"}
    parts = [f"ham {len(terms)}"]
    for coeff, word, wires in terms:
        factors = [f"named {names[c]} {w}" for c, w in zip(word, wires)]
        parts.append(f"{float(coeff)!r} prod {len(factors)} " + " ".join(factors))
    return " ".join(parts)


class Oracle:
    def __init__(self, kind: str = "orc"):
        self.kind = kind
        self.lib = _load(kind)
        self._p = kind + "_"

    def _fn(self, name):
        return getattr(self.lib, self._p + name)

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self._fn("last_error")().decode())

    def num_threads(self) -> int:
        return int(self._fn("num_threads")())

    def sv(self, num_qubits: int, dtype=np.complex128) -> "OracleSV":
        return OracleSV(self, num_qubits, np.dtype(dtype))


class OracleSV:
    def __init__(self, orc: Oracle, n: int, dtype: np.dtype):
        self.o = orc
        self.n = n
        self.dtype = dtype
        self.h = orc._fn("sv_new")(n, 1 if dtype == np.complex128 else 0)
        if not self.h:
            raise RuntimeError(orc._fn("last_error")().decode())

    def __del__(self):
        try:
            self.o._fn("sv_free")(self.h)
        except Exception:
            pass

    # state ---------------------------------------------------------------
    def set_state(self, state):
        s = np.ascontiguousarray(np.asarray(state, dtype=self.dtype))
        assert s.size == 1 << self.n
        self.o._check(self.o._fn("sv_set_state")(self.h, s.ctypes.data_as(C.c_void_p)))

    def state(self) -> np.ndarray:
        out = np.empty(1 << self.n, dtype=self.dtype)
        self.o._check(self.o._fn("sv_get_state")(self.h, out.ctypes.data_as(C.c_void_p)))
        return out

    def set_basis_state(self, bits, wires):
        b, w = _i64(bits), _i64(wires)
        self.o._check(self.o._fn("sv_set_basis_state")(self.h, _p(b, _I64P), _p(w, _I64P), len(w)))

    # gates ---------------------------------------------------------------
    def apply(self, name, wires, inverse=False, params=(), cwires=(), cvals=()):
        w, cw, cv, ps = _i64(wires), _i64(cwires), _u8(cvals), _f64(params)
        self.o._check(self.o._fn("sv_apply")(self.h, name.encode(), _p(cw, _I64P), _p(cv, _U8P), len(cw),
                                             _p(w, _I64P), len(w), int(inverse), _p(ps, _DP), ps.size))

    def apply_matrix(self, mat, wires, inverse=False, cwires=(), cvals=()):
        m = _c128(mat).view(np.float64)
        w, cw, cv = _i64(wires), _i64(cwires), _u8(cvals)
        self.o._check(self.o._fn("sv_apply_matrix")(self.h, _p(m, _DP), _p(cw, _I64P), _p(cv, _U8P), len(cw),
                                                    _p(w, _I64P), len(w), int(inverse)))

    def apply_sparse(self, indptr, indices, data, wires, cwires=(), cvals=()):
        ip, ix, d = _i64(indptr), _i64(indices), _c128(data).view(np.float64)
        w, cw, cv = _i64(wires), _i64(cwires), _u8(cvals)
        self.o._check(self.o._fn("sv_apply_sparse")(self.h, _p(ip, _I64P), _p(ix, _I64P), _p(d, _DP), ix.size,
                                                    _p(cw, _I64P), _p(cv, _U8P), len(cw), _p(w, _I64P), len(w)))

    def apply_pauli_rot(self, wires, inverse, angle, word):
        w = _i64(wires)
        self.o._check(self.o._fn("sv_apply_pauli_rot")(self.h, _p(w, _I64P), len(w), int(inverse), float(angle),
                                                       word.encode()))

    def apply_generator(self, name, wires, adj=False, cwires=(), cvals=()) -> float:
        w, cw, cv = _i64(wires), _i64(cwires), _u8(cvals)
        out = C.c_double()
        self.o._check(self.o._fn("sv_apply_generator")(self.h, name.encode(), _p(cw, _I64P), _p(cv, _U8P), len(cw),
                                                       _p(w, _I64P), len(w), int(adj), C.byref(out)))
        return out.value

    def collapse(self, wire, branch):
        self.o._check(self.o._fn("sv_collapse")(self.h, int(wire), int(branch)))

    def normalize(self):
        self.o._check(self.o._fn("sv_normalize")(self.h))

    # measurements ----------------------------------------------------------
    def probs(self, wires=None) -> np.ndarray:
        if wires is None:
            out = np.empty(1 << self.n)
            self.o._check(self.o._fn("probs")(self.h, None, -1, _p(out, _DP)))
            return out
        w = _i64(wires)
        out = np.empty(1 << len(w))
        self.o._check(self.o._fn("probs")(self.h, _p(w, _I64P), len(w), _p(out, _DP)))
        return out

    def expval_named(self, name, wires) -> float:
        w = _i64(wires)
        out = C.c_double()
        self.o._check(self.o._fn("expval_named")(self.h, name.encode(), _p(w, _I64P), len(w), C.byref(out)))
        return out.value

    def var_named(self, name, wires) -> float:
        w = _i64(wires)
        out = C.c_double()
        self.o._check(self.o._fn("var_named")(self.h, name.encode(), _p(w, _I64P), len(w), C.byref(out)))
        return out.value

    def expval_matrix(self, mat, wires) -> float:
        m = _c128(mat).view(np.float64)
        w = _i64(wires)
        out = C.c_double()
        self.o._check(self.o._fn("expval_matrix")(self.h, _p(m, _DP), _p(w, _I64P), len(w), C.byref(out)))
        return out.value

    def var_matrix(self, mat, wires) -> float:
        m = _c128(mat).view(np.float64)
        w = _i64(wires)
        out = C.c_double()
        self.o._check(self.o._fn("var_matrix")(self.h, _p(m, _DP), _p(w, _I64P), len(w), C.byref(out)))
        return out.value

    def expval_sparse(self, indptr, indices, data) -> float:
        ip, ix, d = _i64(indptr), _i64(indices), _c128(data).view(np.float64)
        out = C.c_double()
        self.o._check(self.o._fn("expval_sparse")(self.h, _p(ip, _I64P), ip.size, _p(ix, _I64P), _p(d, _DP),
                                                  ix.size, C.byref(out)))
        return out.value

    def expval_obs(self, spec: str, od: ObsData | None = None) -> float:
        od = od or ObsData()
        cd, idd = od.arrays()
        out = C.c_double()
        self.o._check(self.o._fn("expval_obs")(self.h, spec.encode(), _p(cd, _DP), _p(idd, _I64P), C.byref(out)))
        return out.value

    def var_obs(self, spec: str, od: ObsData | None = None) -> float:
        od = od or ObsData()
        cd, idd = od.arrays()
        out = C.c_double()
        self.o._check(self.o._fn("var_obs")(self.h, spec.encode(), _p(cd, _DP), _p(idd, _I64P), C.byref(out)))
        return out.value

    def samples(self, shots, seed, wires=None) -> np.ndarray:
        nw = self.n if wires is None else len(wires)
        out = np.empty(shots * nw, dtype=np.int64)
        if wires is None:
            self.o._check(self.o._fn("samples")(self.h, None, -1, shots, seed, _p(out, _I64P)))
        else:
            w = _i64(wires)
            self.o._check(self.o._fn("samples")(self.h, _p(w, _I64P), len(w), shots, seed, _p(out, _I64P)))
        return out.reshape(shots, nw)

    def mcmc_samples(self, kernel: str, burnin: int, shots: int, seed: int) -> np.ndarray:
        out = np.empty(max(1, shots * self.n), dtype=np.int64)
        self.o._check(self.o._fn("mcmc_samples")(self.h, kernel.encode(), burnin, shots, seed, _p(out, _I64P)))
        return out[: shots * self.n].reshape(shots, self.n)

    @staticmethod
    def _ops_arrays(ops):
        names = (C.c_char_p * max(1, len(ops)))(*[o["name"].encode() for o in ops])
        params = _f64([p for o in ops for p in o.get("params", ())] or [0.0])
        nparams = np.array([len(o.get("params", ())) for o in ops] or [0], dtype=np.int32)
        wires = _i64([w for o in ops for w in o["wires"]] or [0])
        nwires = np.array([len(o["wires"]) for o in ops] or [0], dtype=np.int32)
        inv = _u8([int(o.get("inverse", False)) for o in ops] or [0])
        mats = [(_c128(o["matrix"]) if o.get("matrix") is not None else np.zeros(0, np.complex128)) for o in ops]
        mat_sizes = _i64([m.size for m in mats] or [0])
        mflat = np.ascontiguousarray((np.concatenate(mats) if sum(m.size for m in mats) else np.zeros(1, np.complex128)).view(np.float64))
        cw = _i64([w for o in ops for w in o.get("cwires", ())] or [0])
        ncw = np.array([len(o.get("cwires", ())) for o in ops] or [0], dtype=np.int32)
        cv = _u8([int(v) for o in ops for v in o.get("cvals", ())] or [0])
        return (names, _p(params, _DP), nparams.ctypes.data_as(_IP), _p(wires, _I64P), nwires.ctypes.data_as(_IP),
                _p(inv, _U8P), _p(mflat, _DP), _p(mat_sizes, _I64P), _p(cw, _I64P), ncw.ctypes.data_as(_IP),
                _p(cv, _U8P)), (params, nparams, wires, nwires, inv, mflat, mat_sizes, cw, ncw, cv)

    def vjp(self, ops, dy, trainable, apply_ops=False) -> np.ndarray:
        """VectorJacobianProduct: w_j = <dy| d psi / d theta_j> (complex), ops as for adjoint."""
        args, keep = self._ops_arrays(ops)
        d = np.ascontiguousarray(np.asarray(dy, dtype=np.complex128).reshape(-1))
        tp = _i64(trainable or [0])
        out = np.zeros(2 * max(1, len(trainable)))
        self.o._check(self.o._fn("vjp")(self.h, len(ops), *args, _p(d.view(np.float64), _DP), _p(tp, _I64P),
                                        len(trainable), int(apply_ops), _p(out, _DP)))
        del keep
        return out[: 2 * len(trainable)].view(np.complex128).copy()

    def adjoint(self, ops, obs_specs, trainable, od: ObsData | None = None, apply_ops=False) -> np.ndarray:
        """ops: list of dicts {name, params, wires, inverse, matrix, cwires, cvals}."""
        od = od or ObsData()
        names = (C.c_char_p * len(ops))(*[o["name"].encode() for o in ops])
        params = _f64([p for o in ops for p in o.get("params", ())] or [0.0])
        nparams = np.array([len(o.get("params", ())) for o in ops], dtype=np.int32)
        wires = _i64([w for o in ops for w in o["wires"]] or [0])
        nwires = np.array([len(o["wires"]) for o in ops], dtype=np.int32)
        inv = _u8([int(o.get("inverse", False)) for o in ops])
        mats = [(_c128(o["matrix"]) if o.get("matrix") is not None else np.zeros(0, np.complex128)) for o in ops]
        mat_sizes = _i64([m.size for m in mats])
        mflat = np.ascontiguousarray((np.concatenate(mats) if sum(m.size for m in mats) else np.zeros(1, np.complex128)).view(np.float64))
        cw = _i64([w for o in ops for w in o.get("cwires", ())] or [0])
        ncw = np.array([len(o.get("cwires", ())) for o in ops], dtype=np.int32)
        cv = _u8([int(v) for o in ops for v in o.get("cvals", ())] or [0])
        specs = (C.c_char_p * len(obs_specs))(*[s.encode() for s in obs_specs])
        cd, idd = od.arrays()
        tp = _i64(trainable or [0])
        out = np.zeros(max(1, len(obs_specs) * len(trainable)))
        self.o._check(self.o._fn("adjoint")(
            self.h, len(ops), names, _p(params, _DP), nparams.ctypes.data_as(_IP), _p(wires, _I64P),
            nwires.ctypes.data_as(_IP), _p(inv, _U8P), _p(mflat, _DP), _p(mat_sizes, _I64P), _p(cw, _I64P),
            ncw.ctypes.data_as(_IP), _p(cv, _U8P), len(obs_specs), specs, _p(cd, _DP), _p(idd, _I64P),
            _p(tp, _I64P), len(trainable), int(apply_ops), _p(out, _DP)))
        return out[: len(obs_specs) * len(trainable)].reshape(len(obs_specs), len(trainable))
