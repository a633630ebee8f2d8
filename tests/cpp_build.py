"""Compile the C++ test programs under tests/cpp against the built backend
library (or, for the CPU build of the Catalyst device test, against the
oracle-backed test double of its C ABI) and the CPU oracle (test
infrastructure)."""
import shutil
import subprocess
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent
CPP = REPO / "tests" / "cpp"
SRC = CPP / "test_cpp_api.cpp"
LIBDIR = REPO / "pennylane-lightning_gb300" / "lightning_gb300"
ORACLE = REPO / "oracle"


def cxx() -> str:
    for c in ("g++", "c++"):
        if shutil.which(c):
            return c
    raise RuntimeError("no C++ compiler")


def _base(sources) -> list[str]:
    return [cxx(), "-std=c++20", "-O1", "-Wall", "-Wextra", f"-I{REPO / 'include'}", f"-I{ORACLE}",
            *[str(s) for s in sources]]


def _backend_libs() -> list[str]:
    return [f"-L{LIBDIR}", "-l:libplgb300.so", f"-Wl,-rpath,{LIBDIR}"]


def _oracle_libs() -> list[str]:
    return [f"-L{ORACLE}", "-l:liboracle.so", f"-Wl,-rpath,{ORACLE}"]


def compile_cmd(out: Path, syntax_only: bool = False, sources=(SRC,)) -> list[str]:
    cmd = _base(sources)
    if syntax_only:
        return cmd + ["-fsyntax-only"]
    return cmd + ["-o", str(out)] + _backend_libs() + _oracle_libs()


def _run(cmd: list[str], out: Path) -> Path:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(proc.stdout + proc.stderr)
    return out


def build(out: Path, sources=(SRC,)) -> Path:
    """A test program linked against libplgb300.so and liboracle.so."""
    return _run(compile_cmd(out, sources=sources), out)


def build_with_test_double(out: Path, sources) -> Path:
    """A test program linked against the oracle-backed test double of the C
    ABI (tests/cpp/fake_plgb_oracle.cpp) instead of libplgb300.so: runs on
    the CPU."""
    return _run(_base([*sources, CPP / "fake_plgb_oracle.cpp"]) + ["-o", str(out)] + _oracle_libs(), out)


def build_host_only(out: Path, sources) -> Path:
    """A test program that uses only host-side code of the headers."""
    return _run(_base(sources) + ["-o", str(out)], out)
