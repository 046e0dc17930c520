"""In-tree build of the CUDA library ``libmfc_gpu.so`` for sm_103a.

Each translation unit is compiled by its own ``nvcc`` process in parallel,
then linked into one shared library next to this file.  Nothing is installed
into site-packages, so the loaded library is always the in-tree one.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmfc_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]


def unit_flags(src: str) -> list[str]:
    """Per-unit flags.  The plain FP64 path is bit-faithful to the CPU
    reference's operation order, so its device code is compiled without FMA
    contraction (-fmad=false); host code never contracts (-ffp-contract=off,
    which matters on aarch64 hosts where GCC contracts by default).  The
    split-precision units use the approximate FP32 division and square root
    (their FP32 results are checked against the FP64 oracle at a stated
    tolerance).  They are compiled without automatic contraction as well and
    write their fused multiply-adds out as fmaf: contraction left to the
    compiler depends on the surrounding code, so two tile shapes or two code
    paths of one kernel could round the same cell differently."""
    if src.endswith("_fp32.cu"):
        return ["-prec-div=false", "-prec-sqrt=false", "-ftz=true", "-fmad=false"]
    if src.endswith("_fp64fma.cu"):
        # the opt-in contracted FP64 variant (MFC_PREC_FP64_FMA)
        return ["-fmad=true"]
    return ["-fmad=false"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmfc_gpu.so")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps() -> list[str]:
    out = [os.path.abspath(__file__)]
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cu", ".cuh", ".h"))]
    return out


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    flags = FLAGS + (extra_flags or [])

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *flags, *unit_flags(src), "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
