"""The C++ API (include/pl_gb300.hpp: StateVectorGB300, MeasurementsGB300,
observables, OpsData / JacobianData, AdjointJacobianGB300) as a compiled C++
program on the GPU, checked against the CPU oracle inside the program."""
import subprocess

import pytest

from cpp_build import build

pytestmark = pytest.mark.gpu


def test_cpp_api_program(tmp_path):
    from oracle.build_oracle import build_restatement

    build_restatement()
    exe = build(tmp_path / "test_cpp_api")
    proc = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0 and "PASS" in proc.stdout, proc.stdout + proc.stderr
