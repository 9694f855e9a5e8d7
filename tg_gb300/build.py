"""Build recipe of libtgx.so (the C-ABI library) -- nvcc for sm_103a plus gcc.

The CUDA sources are compiled for sm_103a only, with -fmad=false so no FMA
contraction can change a parity-critical result (the kernels also spell those
operations with round-to-nearest intrinsics).  Host C sources are compiled
with -ffp-contract=off for the same reason.  Translation units compile in
parallel; the output lands next to this file (tg_gb300/libtgx.so).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libtgx.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math", "-I", str(ROOT / "include")]
CC_FLAGS = ["-std=gnu11", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall",
            "-I", str(ROOT / "include")]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def sources() -> tuple[list[Path], list[Path]]:
    return sorted(CSRC.glob("*.cu")), sorted(CSRC.glob("*.c"))


def build(verbose: bool = False, extra_nvcc: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    cu, c = sources()
    jobs = []
    objs = []
    for src in cu:
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *(extra_nvcc or []), "-c", str(src), "-o", str(obj)])
    for src in c:
        obj = BUILD / (src.stem + ".c.o")
        objs.append(obj)
        jobs.append(["gcc", *CC_FLAGS, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lgomp", "-lcudart"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra_nvcc=sys.argv[1:])
