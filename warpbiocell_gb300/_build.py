"""Build recipe for libwbc_gb300.so (the sm_103a kernels behind the C-ABI in include/wbc.h).

Each translation unit is compiled by its own nvcc process, in parallel, then linked into one
shared library in ``warpbiocell_gb300/_lib``. The CUDA runtime is linked statically so the
library only needs the driver at run time.

Flags: ``-fmad=false`` keeps every float expression rounding exactly as written (no
multiply-add contraction); with IEEE division and square root (nvcc's defaults) this is what
makes the kernels reproduce the CPU oracle bit for bit.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE_DIR = Path(__file__).resolve().parent
CSRC = PACKAGE_DIR / "csrc"
LIB_DIR = PACKAGE_DIR / "_lib"
LIB_NAME = "libwbc_gb300.so"
SOURCES = ("wbc_runtime.cu", "wbc_mechanics.cu", "wbc_fields.cu", "wbc_cells.cu", "wbc_network.cu", "wbc_sor.cu",
           "wbc_batch.cu", "wbc_adjoint.cu", "wbc_steps.cu")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path() -> str:
    nvcc = shutil.which("nvcc")
    if nvcc is None:
        cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
        if cand.exists():
            nvcc = str(cand)
    if nvcc is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwbc_gb300")
    return nvcc


def common_flags() -> list[str]:
    return [
        ARCH,
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-fmad=false",
        "-Xcompiler",
        "-fPIC",
        "-Xcompiler",
        "-ffp-contract=off",
        f"-I{PACKAGE_DIR.parent / 'include'}",
    ]


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def library_path() -> Path:
    return LIB_DIR / LIB_NAME


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile every .cu in parallel and link libwbc_gb300.so; returns its path."""
    nvcc = nvcc_path()
    obj_dir = LIB_DIR / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    flags = common_flags() + list(extra_flags or [])
    jobs = []
    for src in SOURCES:
        obj = obj_dir / (Path(src).stem + ".o")
        jobs.append(([nvcc, *flags, "-c", str(CSRC / src), "-o", str(obj)], obj))
    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as pool:
        list(pool.map(lambda job: _run(job[0]), jobs))
    out = library_path()
    tmp = out.with_suffix(".so.tmp")
    _run([nvcc, ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *[str(o) for _, o in jobs]])
    os.replace(tmp, out)
    if verbose:
        print(f"built {out}")
    return out
