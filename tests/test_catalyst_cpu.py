"""The Catalyst device (include/pl_gb300_catalyst.hpp) on the CPU: its
host-only parts (keyword parser, DataView, qubit map, subsystem purity,
Hermitian eigen-decomposition), and the whole device test program linked
against an oracle-backed test double of the C ABI, which exercises the
device's host logic (qubit allocation, release, reuse and register
reduction, tape, observable cache, shot handling, mid-circuit measurement,
gradient bookkeeping) without a GPU.  The same program runs against the GPU
library under -m gpu (test_gpu_catalyst.py)."""
import subprocess

from cpp_build import CPP, build_host_only, build_with_test_double


def test_catalyst_host_parts(tmp_path):
    exe = build_host_only(tmp_path / "test_catalyst_host", [CPP / "test_catalyst_host.cpp"])
    proc = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0 and "PASS" in proc.stdout, proc.stdout + proc.stderr


def test_catalyst_device_on_the_test_double(tmp_path):
    from oracle.build_oracle import build_restatement

    build_restatement()
    exe = build_with_test_double(tmp_path / "test_catalyst_device_cpu", [CPP / "test_catalyst_device.cpp"])
    proc = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0 and "PASS" in proc.stdout, proc.stdout + proc.stderr
