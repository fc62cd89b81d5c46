"""Builds the GB300 euler2d library in-tree: euler2d_kokkos_gb300/_build/libe2d_gb300.so
(and the euler2d_gb300 command-line driver beside it).

Translation units compile in parallel, one -gencode for sm_103a.  The FP64
kernels are built with --fmad=false and host code with -ffp-contract=off so
that no multiply-add is contracted: their results are bit-identical to the
reference's FP64 arithmetic.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libe2d_gb300.so")
CLI = os.path.join(OUT, "euler2d_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction either (aarch64 hosts would otherwise fuse
# a*b + c in the parameter and ring-geometry arithmetic)
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

# (source, extra nvcc flags)
UNITS = [
    ("e2d_fp64.cu", ["--fmad=false"]),
    ("e2d_fp32c.cu", ["-use_fast_math"]),
    ("e2d_reduce.cu", ["--fmad=false"]),
    ("e2d_probe.cu", ["--fmad=false"]),
    ("e2d_impl12.cu", ["--fmad=false"]),
    ("e2d_noalloc.cu", []),
    ("e2d_batch.cu", []),
    ("e2d_capi.cu", []),
    ("e2d_config.cpp", ["-x", "cu"]),
]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libe2d_gb300.so")


def _compile(src: str, extra: list[str], verbose_ptxas: bool) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas and src.endswith(".cu"):
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile every CUDA unit for sm_103a and link the shared library."""
    os.makedirs(OUT, exist_ok=True)
    units = [(s, f) for s, f in UNITS if os.path.exists(os.path.join(CSRC, s))]
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "e2d.h")]
    if not force and not _stale(LIB, deps) and not _stale(CLI, deps):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(units) + 1) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose_ptxas), units))
    link = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    main_src = os.path.join(CSRC, "euler2d_main.cpp")
    if os.path.exists(main_src):
        cmd = [nvcc(), *ARCH, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
               "-x", "cu", main_src, "-o", CLI, "-L" + OUT, "-le2d_gb300",
               "-Xlinker", "-rpath=$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
