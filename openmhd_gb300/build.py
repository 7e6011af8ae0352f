"""Build libopenmhd_gb300.so (sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel; units that must reproduce the
reference's IEEE-754 operation sequence are compiled with --fmad=false.
Usage: python -m openmhd_gb300.build [--force] [--verbose]
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
LIB = os.path.join(HERE, "libopenmhd_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]

# translation unit -> extra flags
UNITS = {
    "omhd_runtime.cu": [],
    "omhd_routines.cu": ["--fmad=false"],
    "omhd_solver.cu": [],
    "omhd_fused2d_fp64.cu": ["--fmad=true"],
    "omhd_fused2d_parity.cu": ["--fmad=false"],
    "omhd_fused2d_mixed.cu": ["--fmad=true"],
    "omhd_fused3d_fp64.cu": ["--fmad=true"],
    "omhd_fused3d_parity.cu": ["--fmad=false"],
    "omhd_fused3d_mixed.cu": ["--fmad=true"],
    "omhd_noalloc.cu": [],
    "omhd_ensemble.cu": [],
    "omhd_adjoint.cu": ["--fmad=true"],
    "omhd_fileio.cu": [],
}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build openmhd_gb300")
    return cand


def _deps_newer(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    heads = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    heads.append(os.path.join(HERE, "..", "include", "openmhd_gb300.h"))
    return any(os.path.getmtime(p) > t for p in [src] + heads)


def _compile(unit: str, flags: list[str], force: bool, verbose: bool, extra: list[str]) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
    if force or _deps_newer(obj, src):
        cmd = [nvcc()] + ARCH + COMMON + flags + extra + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stderr.strip() or r.stdout.strip()):
            print(r.stdout + r.stderr, flush=True)
    return obj


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, u, f, force, verbose, extra) for u, f in UNITS.items()]
        objs = [f.result() for f in futs]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
