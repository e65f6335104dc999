"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/wbc_oracle.cpp`` into ``oracle/_build/liboracle.so`` with g++, OpenMP and
``-ffp-contract=off`` (no fused multiply-add, so float expressions round exactly as written, as
in the GPU library compiled with ``-fmad=false``). No architecture-specific flags: the same
source gives the same results on x86-64 and aarch64.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
LIB = BUILD_DIR / "liboracle.so"
SOURCE = ORACLE_DIR / "wbc_oracle.cpp"


def build(force: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime >= SOURCE.stat().st_mtime:
        return LIB
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("g++ not found: cannot build the oracle")
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(f".so.{os.getpid()}.tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           str(SOURCE), "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
