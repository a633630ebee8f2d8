"""Compile the C++ API test program (tests/cpp/test_cpp_api.cpp) against the
built backend library and the CPU oracle (test infrastructure)."""
import shutil
import subprocess
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent
SRC = REPO / "tests" / "cpp" / "test_cpp_api.cpp"
LIBDIR = REPO / "pennylane-lightning_gb300" / "lightning_gb300"
ORACLE = REPO / "oracle"


def cxx() -> str:
    for c in ("g++", "c++"):
        if shutil.which(c):
            return c
    raise RuntimeError("no C++ compiler")


def compile_cmd(out: Path, syntax_only: bool = False) -> list[str]:
    cmd = [cxx(), "-std=c++20", "-O1", "-Wall", "-Wextra", f"-I{REPO / 'include'}", f"-I{ORACLE}", str(SRC)]
    if syntax_only:
        return cmd + ["-fsyntax-only"]
    return cmd + ["-o", str(out), f"-L{LIBDIR}", "-l:libplgb300.so", f"-L{ORACLE}", "-l:liboracle.so",
                  f"-Wl,-rpath,{LIBDIR}", f"-Wl,-rpath,{ORACLE}"]


def build(out: Path) -> Path:
    proc = subprocess.run(compile_cmd(out), capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(proc.stdout + proc.stderr)
    return out
