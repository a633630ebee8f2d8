"""GB300-native (sm_103a) state-vector backend with lightning.qubit's API.

``lightning_gb300_ops`` mirrors the reference's ``lightning_qubit_ops``
binding module; everything runs through the C ABI of include/pl_gb300.h.
"""
from . import lightning_gb300_ops
from ._capi import LIB_PATH, LightningException

__all__ = ["lightning_gb300_ops", "LightningException", "LIB_PATH"]
