"""Builds the oracle (test infrastructure only).

- liboracle.so: the C++ restatement (mat_oracle.cpp), built here and on the
  GPU host (portable flags; FMA is explicit std::fma so results are
  identical on x86-64 and aarch64).
- _ref/libmatref.so: the reference Mat-8.3.1 compiled from its own headers
  with ref_shim/ (only where the reference tree exists; x86-64 AVX-512 build,
  Mat's configuration for its published numbers).
- _ref/libmat81ref.so: the Mat-8.1 snapshot's EVD_Q tridiagonalisation and QR
  iteration compiled from its own headers with ref81_shim/ (same conditions).
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
REF_LIB = REF_DIR / "libmatref.so"
# The reference tree (read only; absent on the GPU host).  MAT_REFERENCE_ROOT
# overrides where it is looked for.
REFERENCE_TREE = Path(os.environ.get("MAT_REFERENCE_ROOT", "/root/reference"))
REFERENCE_ROOT = REFERENCE_TREE / "Mat-8.3.1"
REF81_LIB = REF_DIR / "libmat81ref.so"
REFERENCE81_ROOT = REFERENCE_TREE / "Mat-8.1"
# the seeded input streams the oracle shares with the library
RNG_HEADER = HERE.parent / "mat_gb300" / "csrc" / "rng.cuh"


def _cxx() -> str:
    return os.environ.get("CXX", "g++")


def _arch_flags() -> list[str]:
    # hardware FMA for std::fma on x86-64 (aarch64 has it in the base ISA)
    return ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []


def _stale(lib: Path, deps: list[Path]) -> bool:
    return not lib.exists() or any(d.stat().st_mtime > lib.stat().st_mtime for d in deps)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "mat_oracle.cpp"
    if force or _stale(ORACLE_LIB, [src, RNG_HEADER, Path(__file__)]):
        cmd = [_cxx(), "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
               *_arch_flags(), str(src), "-o", str(ORACLE_LIB)]
        subprocess.run(cmd, check=True)
    return ORACLE_LIB


def build_ref(force: bool = False) -> Path | None:
    """Compiles the reference (only where its headers exist and the host is x86-64 with AVX-512)."""
    if not REFERENCE_ROOT.exists() or platform.machine() not in ("x86_64", "AMD64"):
        return None
    src = HERE / "ref_wrap.cpp"
    deps = [src, *sorted((HERE / "ref_shim").rglob("*.h")), Path(__file__)]
    if force or _stale(REF_LIB, deps):
        REF_DIR.mkdir(exist_ok=True)
        cmd = [_cxx(), "-O3", "-std=c++17", "-fPIC", "-shared", "-D__AVX512__", "-mavx512f", "-mavx512dq",
               "-mavx512vl", "-mfma", "-I", str(HERE / "ref_shim"), "-I", str(HERE / "ref_shim" / "QR"),
               "-I", str(REFERENCE_ROOT), str(src), "-o", str(REF_LIB)]
        subprocess.run(cmd, check=True)
    return REF_LIB


def build_ref81(force: bool = False) -> Path | None:
    """Compiles the Mat-8.1 snapshot's EVD_Q tridiagonalisation and QR iteration (ref81_wrap.cpp)."""
    if not REFERENCE81_ROOT.exists() or platform.machine() not in ("x86_64", "AMD64"):
        return None
    src = HERE / "ref81_wrap.cpp"
    deps = [src, *sorted((HERE / "ref81_shim").rglob("*.h")), Path(__file__)]
    if force or _stale(REF81_LIB, deps):
        REF_DIR.mkdir(exist_ok=True)
        cmd = [_cxx(), "-O3", "-std=c++17", "-fPIC", "-shared", "-D__AVX512__", "-mavx512f", "-mavx512dq",
               "-mavx512vl", "-mfma", "-I", str(HERE / "ref81_shim"), "-I", str(REFERENCE81_ROOT), str(src),
               "-o", str(REF81_LIB)]
        subprocess.run(cmd, check=True)
    return REF81_LIB


def build(force: bool = False, verbose: bool = False) -> None:
    o = build_oracle(force)
    r = build_ref(force)
    build_ref81(force)
    if verbose:
        print(f"built {o}" + (f" and {r}" if r else " (reference tree absent: no _ref build)"), file=sys.stderr)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
