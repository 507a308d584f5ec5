"""Builds the CUDA library (weldformfem_gb300/_lib/libwf_gb300.so) in-tree.

One nvcc invocation per translation unit, run in parallel, for sm_103a only;
the library links the CUDA runtime statically and exports only the C ABI of
include/wf.h. The FP64 kernels are compiled with --fmad=false so that they
round exactly as the reference CPU code (built without FMA contraction).
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
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB_PATH = os.path.join(OUT_DIR, "libwf_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                 f"-I{os.path.join(ROOT, 'include')}", f"-I{CSRC}"]
UNITS = {
    "wf_api.cu": ["-Xcompiler", "-ffp-contract=off"],
    "wf_fp64.cu": ["--fmad=false"],
    "wf_mixed.cu": [],
    "wf_reduce.cu": [],
    "wf_setup.cu": [],
    "wf_noalloc.cu": ["--fmad=false"],
    "wf_adjoint.cu": [],
    "wf_deck.cpp": ["-Xcompiler", "-ffp-contract=off"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, u) for u in UNITS] + [
        os.path.join(CSRC, "wf_internal.cuh"), os.path.join(CSRC, "wf_adjoint.cuh"),
        os.path.join(CSRC, "wf_trimesh.cuh"),
        os.path.join(ROOT, "include", "wf.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False, extra: list | None = None) -> str:
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    nv = nvcc()
    extra = list(extra or [])

    def compile_one(unit):
        obj = os.path.join(OBJ_DIR, os.path.splitext(unit)[0] + ".o")
        cmd = [nv] + COMMON + UNITS[unit] + extra + ["-c", os.path.join(CSRC, unit), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB_PATH + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
