"""Builds libhystrath_gb300.so in-tree with nvcc for sm_103a.

Translation units compile in parallel; the result lands in
hystrath_gb300/_build/.  The library has no CPU path: on a machine without a
GB300 it loads, but dsmc_create_from_spec reports DSMC_ERR_NO_DEVICE.
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
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libhystrath_gb300.so")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
# dsmc_move.cu must not contract a*b+c into fma: the CPU replay evaluates the
# same move, crossing and index expressions operation by operation and the two
# agree bit for bit.  Collisions and sampling agree statistically, so
# dsmc_collide.cu lets the compiler fuse.
UNITS = {
    "dsmc_move.cu": ["-fmad=false"],
    "dsmc_collide.cu": [],
    "dsmc_api.cu": [],
    "dsmc_noalloc.cu": [],
    "dsmc_mlp.cu": [],
    "case_parser.cpp": [],
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    # host code must not contract either (aarch64 GCC contracts by default)
    cmd = [_nvcc(), GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", src, "-o", obj] + extra
    if src.endswith(".cpp"):
        cmd = [_nvcc(), "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-x", "c++",
               "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = {os.path.join(CSRC, k): v for k, v in UNITS.items()}
    newest = max(os.path.getmtime(p) for p in list(srcs) +
                 [os.path.join(CSRC, f) for f in os.listdir(CSRC)] +
                 [os.path.join(ROOT, "include", "hystrath_gb300.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), srcs.items()))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), GENCODE, "-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
