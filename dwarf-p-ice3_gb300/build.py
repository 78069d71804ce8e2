"""Build libice3gb.so in-tree with nvcc for sm_103a (GB300).

    python dwarf-p-ice3_gb300/build.py [--force] [--verbose]

Each .cu is compiled in parallel (one -gencode, -lineinfo), then linked into
dwarf-p-ice3_gb300/lib/libice3gb.so with the CUDA runtime linked statically.
Extra nvcc flags (e.g. -D switches of the kernels) can be given in the
ICE3GB_NVCC_FLAGS environment variable; use --force after changing them.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(LIB_DIR, "libice3gb.so")
INCLUDE = os.path.normpath(os.path.join(HERE, "..", "include"))
SOURCES = ["ice_adjust.cu", "ice_adjust_vjp.cu", "sedimentation.cu", "sedimentation_vjp.cu", "rain_ice.cu",
           "rain_ice_ts.cu", "mlp.cu", "surrogate.cu", "surrogate_rain_ice.cu", "abi.cu", "rain_ice_noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    return files + [os.path.join(INCLUDE, "ice3gb.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        extra = os.environ.get("ICE3GB_NVCC_FLAGS", "").split()
        cmd = [cc, *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
