"""Build libhycadv.so in-tree with nvcc for sm_103a (GB300).

Translation units are compiled in parallel into ``_build/`` and linked into
``hycadv/_lib/libhycadv.so`` with the CUDA runtime linked statically, so the
library needs only the driver (libcuda) at run time.
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
LIBDIR = os.path.join(HERE, "hycadv", "_lib")
LIB = os.path.join(LIBDIR, "libhycadv.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]

# translation unit -> extra flags.  The FP64 kernels are built without FMA
# contraction so that every operation rounds as in the reference build.
UNITS = {
    "hyc_fp64.cu": ["-lineinfo", "-fmad=false"],
    "hyc_fct2c.cu": ["-lineinfo", "-fmad=false"],
    "hyc_tsdff.cu": ["-lineinfo", "-fmad=false"],
    "hyc_asselin.cu": ["-lineinfo", "-fmad=false"],
    "hyc_cnuity.cu": ["-lineinfo", "-fmad=false"],
    "hyc_host.cpp": [],
    "hyc_noalloc.cu": ["-lineinfo"],
    "hyc_mixed_col2.cu": ["-lineinfo"],
    "hyc_ens_util.cu": ["-lineinfo"],
    "hyc_ens_host.cpp": [],
    "hyc_za.cpp": [],
    "hyc_tmap.cpp": [],
}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out.append(os.path.join(INCLUDE, "hycom_adv.h"))
    return out


def _compile(src: str, flags: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
