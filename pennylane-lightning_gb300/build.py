"""Build the GB300 backend library in-tree.

Compiles every translation unit of ``csrc/`` with nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and links
``lightning_gb300/libplgb300.so`` next to the Python binding that loads it.
No cmake, no torch extension machinery: the library is a plain C-ABI shared
object (include/pl_gb300.h).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "lightning_gb300"
BUILD = PKG / "_build"
LIB = OUT_DIR / "libplgb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (CUDA toolkit required to build the GB300 backend)")


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def flags() -> list[str]:
    return [
        *ARCH,
        "-O3",
        "-lineinfo",
        "-std=c++20",
        "--expt-relaxed-constexpr",
        "-Xcompiler", "-fPIC",
        "-Xcompiler", "-O3",
        "-Xptxas", "-O3",
        f"-I{REPO / 'include'}",
        f"-I{CSRC}",
    ]


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    deps = [src, *CSRC.glob("*.hpp"), *CSRC.glob("*.cuh"), *(REPO / "include").glob("*.h")]
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path) -> Path:
    obj = BUILD / (src.name + ".o")
    if _stale(obj, src):
        cmd = [nvcc(), *flags(), "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cpp":
            cmd = [nvcc(), *flags(), "-x", "cu", "-c", str(src), "-o", str(obj)]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{proc.stdout}\n{proc.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(_compile, srcs))
    if not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{proc.stdout}\n{proc.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
