"""CPU checks of the C ABI library (no GPU needed): it loads, it exports every
symbol include/pl_gb300.h declares, module-level info works, and without a
GPU a state vector cannot be created (the backend fails loudly instead of
falling back to the CPU)."""
import ctypes as C
import re
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (REPO / "include").glob("*.h"):
        txt = h.read_text()
        names |= set(re.findall(r"^\s*(?:int|const char \*)\s*(plgb_\w+)\s*\(", txt, flags=re.M))
    return sorted(names)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert len(syms) >= 45
    assert "plgb_sv_apply_operation" in syms and "plgb_adjoint_jacobian" in syms


def test_library_exports_all_declared_symbols():
    from lightning_gb300 import _capi

    lib = _capi.lib()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # and the Python binding binds exactly the declared set
    assert set(_capi.SIGNATURES) == set(declared_symbols())


def test_module_info(ops_module):
    assert ops_module.backend_info()["NAME"] == "lightning.gb300"
    info = ops_module.runtime_info()
    assert info["compiled_for"] == "sm_103a"
    a = ops_module.allocate_aligned_array(100, "complex128", True)
    assert a.size == 100 and a.ctypes.data % 64 == 0 and not a.any()


def test_no_cpu_fallback_without_gpu(ops_module):
    from lightning_gb300 import _capi

    count = C.c_int()
    _capi.call("plgb_device_count", C.byref(count))
    if count.value > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="no GPU"):
        ops_module.StateVectorC128(3)


def test_invalid_arguments_are_rejected_on_the_host(ops_module):
    from lightning_gb300 import _capi

    h = C.c_void_p()
    rc = _capi.lib().plgb_sv_create(3, 96, C.byref(h))
    assert rc == 1 and b"precision" in _capi.lib().plgb_last_error()
    with pytest.raises(RuntimeError, match="disjoint"):
        ops_module.observables.TensorProdObsC128([ops_module.observables.NamedObsC128("PauliX", [0]),
                                                  ops_module.observables.NamedObsC128("PauliZ", [0])])
    with pytest.raises(RuntimeError, match="unknown observable"):
        ops_module.observables.NamedObsC128("NotAnObservable", [0])


def test_process_wide_settings_roundtrip(ops_module):
    # lazy fusion default, its qubit threshold and the tile variant are host
    # settings: set, read back through the previous value, restore
    from lightning_gb300 import _capi

    prev = ops_module.set_lazy_min_qubits(20)
    assert ops_module.set_lazy_min_qubits(prev) == 20
    assert _capi.lib().plgb_set_lazy_min_qubits(0) == -1  # rejected, unchanged
    assert ops_module.set_lazy_min_qubits(prev) == prev
    with pytest.raises(ValueError):
        ops_module.set_lazy_min_qubits(0)
    on = ops_module.set_lazy_fusion(False)
    assert ops_module.set_lazy_fusion(on) is False
    assert _capi.lib().plgb_set_tile_variant(32, 1) == -1  # no such precision


def test_cpp_api_header_compiles():
    # include/pl_gb300.hpp (the C++ API) and its test program compile; the
    # program itself runs under -m gpu (test_gpu_cpp_api.py)
    import subprocess

    from cpp_build import compile_cmd

    proc = subprocess.run(compile_cmd(REPO / "unused", syntax_only=True), capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr


def test_catalyst_device_links_against_the_backend(tmp_path):
    # the Catalyst device test program links against libplgb300.so (every C
    # ABI entry point the device calls is exported); it runs under -m gpu
    import subprocess

    from cpp_build import CPP, compile_cmd

    proc = subprocess.run(compile_cmd(tmp_path / "catalyst_link", sources=(CPP / "test_catalyst_device.cpp",)),
                          capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr
