"""Build recipe for the CPU oracles (test infrastructure only).

* ``oracle/liboracle.so`` — this repository's C++ restatement of the
  lightning.qubit LM algorithms (``lm_oracle.cpp``).  Built everywhere
  (x86 container and the aarch64 GPU host) with OpenMP, mirroring the
  reference wheel's ``LQ_ENABLE_KERNEL_OMP=ON`` build.
* ``oracle/_ref/libplref.so`` — ``ref_shim.cpp`` compiled against the
  reference's own headers and ``.cpp`` files *where they lie* under the
  reference checkout (nothing is copied).  Built only when the checkout is
  present; output goes to ``oracle/_ref/`` (git-ignored).

The reference file list and flags follow its CMake setup
(pennylane_lightning/core/simulators/lightning_qubit/gates/CMakeLists.txt:
x86 branch adds the AVX2/AVX512 kernel maps; other hosts use the default map).
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
# the reference checkout: PL_REFERENCE_ROOT, else a "reference" directory
# beside this repository's root
REF_ROOT = Path(os.environ.get("PL_REFERENCE_ROOT", HERE.parent.parent / "reference"))
REF_OUT = HERE / "_ref"

# -ffp-contract=off: no FMA contraction, so the restatement rounds like the
# reference's x86 build (which has no FMA unit enabled) on every host.
CXXFLAGS = ["-std=c++20", "-O3", "-DNDEBUG", "-fPIC", "-fopenmp", "-ffp-contract=off"]


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build_restatement(force: bool = False) -> Path:
    out = HERE / "liboracle.so"
    deps = [HERE / "lm_oracle.cpp", HERE / "lm_oracle.hpp", HERE / "obs_spec.hpp", HERE / "oracle_api.h"]
    if force or _stale(out, deps):
        _run(["g++", *CXXFLAGS, "-shared", "-o", str(out), str(HERE / "lm_oracle.cpp")])
    return out


def _ref_include_dirs(core: Path) -> list[str]:
    skip = ("lightning_gpu", "lightning_kokkos", "lightning_tensor", "catalyst", "tests", "bindings")
    dirs = []
    for d, _subdirs, _files in os.walk(core):
        p = Path(d)
        rel = p.relative_to(core).parts
        if any(s in rel for s in skip):
            continue
        dirs.append(f"-I{p}")
    return dirs


def build_reference(force: bool = False) -> Path | None:
    """Compile the reference's lightning.qubit core + ref_shim.cpp into oracle/_ref."""
    core = REF_ROOT / "pennylane_lightning" / "core"
    if not core.is_dir():
        return None
    out = REF_OUT / "libplref.so"
    if not force and out.exists() and not _stale(out, [HERE / "ref_shim.cpp", HERE / "obs_spec.hpp", HERE / "oracle_api.h"]):
        return out
    REF_OUT.mkdir(exist_ok=True)
    lq = core / "simulators" / "lightning_qubit"
    gates = lq / "gates"
    x86 = platform.machine() in ("x86_64", "AMD64")
    defs = ["-DPL_USE_OMP=1", "-DPL_LQ_KERNEL_OMP", "-D_ENABLE_PLQUBIT=1"]
    incs = _ref_include_dirs(core)
    base = CXXFLAGS + defs + incs
    if x86:
        base = base + ["-mavx"]
        srcs = [
            (gates / "KernelMap_X64.cpp", []),
            (gates / "AssignKernelMap_Default.cpp", []),
            (gates / "AssignKernelMap_AVX2.cpp", []),
            (gates / "AssignKernelMap_AVX512.cpp", []),
            (gates / "RegisterKernels_x64.cpp", []),
            (gates / "RegisterKernels_AVX2.cpp", ["-mavx2", "-mfma"]),
            (gates / "RegisterKernels_AVX512.cpp", ["-mavx512f"]),
        ]
    else:
        srcs = [
            (gates / "KernelMap_Default.cpp", []),
            (gates / "AssignKernelMap_Default.cpp", []),
            (gates / "RegisterKernels_Default.cpp", []),
        ]
    srcs += [
        (gates / "GateIndices.cpp", []),
        (gates / "cpu_kernels" / "GateImplementationsLM.cpp", []),
        (core / "utils" / "RuntimeInfo.cpp", []),
        (HERE / "ref_shim.cpp", [f"-I{HERE}"]),
    ]
    objs = []

    def compile_one(item):
        src, extra = item
        obj = REF_OUT / (src.stem + ".o")
        _run(["g++", *base, *extra, "-c", str(src), "-o", str(obj)])
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    _run(["g++", "-shared", "-fopenmp", "-o", str(out), *map(str, objs)])
    return out


def main() -> int:
    print(build_restatement(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
    return 0


if __name__ == "__main__":
    sys.exit(main())
