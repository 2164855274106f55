"""Build the sm_103a shared library of the solve step (in-tree, no cmake).

Every .cu file of fast_gb300/csrc is compiled in parallel with

    nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo --fmad=false

and linked into fast_gb300/_lib/libfastgb300.so.  ``--fmad=false`` keeps every
FP64 multiply and add separately rounded (the reference's arithmetic);
``-ffp-contract=off`` does the same for the host-side constant evaluation
(aarch64 compilers contract by default).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "libfastgb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "--fmad=false", "-std=c++17",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-Xptxas", "-warn-spills",
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fast_gb300")
    return exe


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    cmd = [nvcc(), *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile the CUDA sources if any is newer than the library; return its path."""
    extra = extra or []
    OUT_DIR.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    deps = srcs + sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "fast_gb300.h"]
    if LIB.exists() and not force:
        t_lib = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= t_lib for p in deps):
            return LIB
    objs = [OUT_DIR / (s.stem + ".o") for s in srcs]
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], extra), zip(srcs, objs)))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
