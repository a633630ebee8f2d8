"""The Catalyst device (include/pl_gb300_catalyst.hpp) as a compiled C++
program on the GPU (libplgb300.so), checked against the CPU oracle and the
reference's device-test known answers inside the program."""
import subprocess

import pytest

from cpp_build import CPP, build

pytestmark = pytest.mark.gpu


def test_catalyst_device_program(tmp_path):
    from oracle.build_oracle import build_restatement

    build_restatement()
    exe = build(tmp_path / "test_catalyst_device", sources=(CPP / "test_catalyst_device.cpp",))
    proc = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(proc.stdout)
    assert proc.returncode == 0 and "PASS" in proc.stdout, proc.stdout + proc.stderr
