"""ctypes loader for the GB300 C ABI (include/pl_gb300.h).

The shared library is built in-tree by ``pennylane-lightning_gb300/build.py``
into this package directory.  Loading fails loudly when it is missing: the
backend has no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libplgb300.so"

I64P = C.POINTER(C.c_int64)
U8P = C.POINTER(C.c_uint8)
DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)
VP = C.c_void_p

# name: (restype, argtypes)
SIGNATURES = {
    "plgb_last_error": (C.c_char_p, []),
    "plgb_backend_info": (C.c_int, [C.c_char_p, C.c_size_t]),
    "plgb_runtime_info": (C.c_int, [C.c_char_p, C.c_size_t]),
    "plgb_device_count": (C.c_int, [IP]),
    "plgb_kernel_launches": (C.c_int, [C.POINTER(C.c_uint64)]),
    "plgb_device_allocations": (C.c_int, [C.POINTER(C.c_uint64)]),
    "plgb_sv_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(VP)]),
    "plgb_sv_create_raw": (C.c_int, [VP, C.c_int, C.c_int, C.POINTER(VP)]),
    "plgb_sv_clone": (C.c_int, [VP, C.POINTER(VP)]),
    "plgb_sv_destroy": (C.c_int, [VP]),
    "plgb_sv_num_qubits": (C.c_int, [VP, IP]),
    "plgb_sv_precision": (C.c_int, [VP, IP]),
    "plgb_sv_length": (C.c_int, [VP, C.POINTER(C.c_uint64)]),
    "plgb_sv_device_ptr": (C.c_int, [VP, C.POINTER(VP)]),
    "plgb_sv_synchronize": (C.c_int, [VP]),
    "plgb_sv_stream": (C.c_int, [VP, C.POINTER(VP)]),
    "plgb_sv_reset": (C.c_int, [VP]),
    "plgb_sv_set_basis_state": (C.c_int, [VP, I64P, I64P, C.c_int]),
    "plgb_sv_set_state_vector": (C.c_int, [VP, VP, C.c_uint64, I64P, C.c_int]),
    "plgb_sv_update_data": (C.c_int, [VP, VP, C.c_uint64]),
    "plgb_sv_get_state": (C.c_int, [VP, VP, C.c_uint64]),
    "plgb_sv_apply_operation": (C.c_int, [VP, C.c_char_p, I64P, C.c_int, C.c_int, DP, C.c_int]),
    "plgb_sv_apply_controlled_operation": (C.c_int, [VP, C.c_char_p, I64P, U8P, C.c_int, I64P, C.c_int, C.c_int,
                                                     DP, C.c_int]),
    "plgb_sv_apply_matrix": (C.c_int, [VP, DP, I64P, C.c_int, C.c_int]),
    "plgb_sv_apply_controlled_matrix": (C.c_int, [VP, DP, I64P, U8P, C.c_int, I64P, C.c_int, C.c_int]),
    "plgb_sv_apply_sparse_matrix": (C.c_int, [VP, I64P, I64P, DP, C.c_int64, I64P, U8P, C.c_int, I64P, C.c_int]),
    "plgb_sv_apply_pauli_rot": (C.c_int, [VP, I64P, C.c_int, C.c_int, C.c_double, C.c_char_p]),
    "plgb_sv_apply_generator": (C.c_int, [VP, C.c_char_p, I64P, U8P, C.c_int, I64P, C.c_int, C.c_int, DP]),
    "plgb_sv_collapse": (C.c_int, [VP, C.c_int64, C.c_int]),
    "plgb_sv_normalize": (C.c_int, [VP]),
    "plgb_meas_probs": (C.c_int, [VP, I64P, C.c_int, DP]),
    "plgb_meas_expval_named": (C.c_int, [VP, C.c_char_p, I64P, C.c_int, DP]),
    "plgb_meas_expval_matrix": (C.c_int, [VP, DP, I64P, C.c_int, DP]),
    "plgb_meas_expval_matrix_noalloc": (C.c_int, [VP, DP, I64P, C.c_int, DP]),
    "plgb_batch_create": (C.c_int, [C.c_int, C.POINTER(VP)]),
    "plgb_batch_destroy": (C.c_int, [VP]),
    "plgb_batch_configure": (C.c_int, [VP, C.c_int, C.c_int64, C.c_int]),
    "plgb_batch_run": (C.c_int, [VP, C.c_int, VP, VP, VP, VP, VP, VP, VP, VP, VP, VP, VP, VP, DP]),
    "plgb_batch_adjoint": (C.c_int, [VP, C.c_int, VP, VP, VP, VP, VP, VP, VP, VP, VP, VP, VP, VP, DP, DP]),
    "plgb_batch_stats": (C.c_int, [VP, C.c_char_p, C.c_size_t]),
    "plgb_gate_name": (C.c_char_p, [C.c_int]),
    "plgb_set_c128_fp64_passes": (C.c_int, [C.c_int]),
    "plgb_set_tc_dense": (C.c_int, [C.c_int]),
    "plgb_sv_apply_operations_blocks": (C.c_int, [VP, VP, C.c_int, C.POINTER(C.c_int)]),
    "plgb_ops_block_plan": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_size_t]),
    "plgb_set_tile_variant": (C.c_int, [C.c_int, C.c_int]),
    "plgb_set_lazy_fusion": (C.c_int, [C.c_int]),
    "plgb_sv_set_lazy": (C.c_int, [VP, C.c_int]),
    "plgb_set_lazy_min_qubits": (C.c_int, [C.c_int]),
    "plgb_meas_expval_sparse": (C.c_int, [VP, I64P, C.c_int64, I64P, DP, C.c_int64, DP]),
    "plgb_meas_expval_obs": (C.c_int, [VP, VP, DP]),
    "plgb_meas_var_obs": (C.c_int, [VP, VP, DP]),
    "plgb_meas_var_named": (C.c_int, [VP, C.c_char_p, I64P, C.c_int, DP]),
    "plgb_meas_var_matrix": (C.c_int, [VP, DP, I64P, C.c_int, DP]),
    "plgb_meas_var_sparse": (C.c_int, [VP, I64P, C.c_int64, I64P, DP, C.c_int64, DP]),
    "plgb_meas_generate_samples": (C.c_int, [VP, I64P, C.c_int, C.c_int64, C.c_uint64, I64P]),
    "plgb_meas_generate_mcmc_samples": (C.c_int, [VP, C.c_char_p, C.c_int64, C.c_int64, C.c_uint64, I64P]),
    "plgb_obs_named": (C.c_int, [C.c_char_p, I64P, C.c_int, C.POINTER(VP)]),
    "plgb_obs_hermitian": (C.c_int, [DP, I64P, C.c_int, C.POINTER(VP)]),
    "plgb_obs_tensor_prod": (C.c_int, [C.POINTER(VP), C.c_int, C.POINTER(VP)]),
    "plgb_obs_hamiltonian": (C.c_int, [DP, C.POINTER(VP), C.c_int, C.POINTER(VP)]),
    "plgb_obs_sparse_hamiltonian": (C.c_int, [DP, I64P, C.c_int64, I64P, C.c_int64, I64P, C.c_int, C.POINTER(VP)]),
    "plgb_obs_destroy": (C.c_int, [VP]),
    "plgb_obs_wires": (C.c_int, [VP, I64P, C.c_int, IP]),
    "plgb_obs_repr": (C.c_int, [VP, C.c_char_p, C.c_size_t]),
    "plgb_ops_create": (C.c_int, [C.c_int, C.POINTER(C.c_char_p), DP, IP, I64P, IP, U8P, DP, I64P, I64P, IP, U8P,
                                  C.POINTER(VP)]),
    "plgb_ops_destroy": (C.c_int, [VP]),
    "plgb_ops_num_par_ops": (C.c_int, [VP, IP]),
    "plgb_sv_apply_operations": (C.c_int, [VP, VP, C.c_int, IP]),
    "plgb_ops_fusion_plan": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_size_t]),
    "plgb_adjoint_jacobian": (C.c_int, [VP, C.POINTER(VP), C.c_int, VP, I64P, C.c_int, C.c_int, DP]),
    "plgb_vjp": (C.c_int, [VP, VP, DP, I64P, C.c_int, DP]),
    "plgb_adjoint_jacobian_inplace": (C.c_int, [VP, C.POINTER(VP), C.c_int, VP, I64P, C.c_int, DP]),
}

_LIB: C.CDLL | None = None


class LightningException(RuntimeError):
    """Error raised by the backend (the reference's LightningException)."""


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"GB300 backend library not built: {LIB_PATH} is missing "
                "(run pennylane-lightning_gb300/build.py); there is no CPU fallback"
            )
        handle = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | getattr(os, "RTLD_LOCAL", 0))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = handle
    return _LIB


def check(rc: int) -> None:
    if rc != 0:
        msg = lib().plgb_last_error()
        raise LightningException(msg.decode() if msg else f"error code {rc}")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
