"""Build ``vmbd_gb300/_lib/libvmbd_eff.so`` (sm_103a) with nvcc, in tree.

One object per translation unit, compiled in parallel, then linked into a
shared library with the CUDA runtime linked statically.  Rebuilds only when a
source or header is newer than the library.

``build(debug=True)`` builds the bounds-checked variant
``libvmbd_eff_debug.so`` (``-DEFF_DEBUG``: every frame and global index the
kernels form is checked and a bad one is recorded in the plan's device error
word instead of being used), with the frame-64 and frame-128 kernels only --
the frames of the small parity fixtures it is run on.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libvmbd_eff.so")
DEBUG_LIB = os.path.join(OUT_DIR, "libvmbd_eff_debug.so")
# translation units left out of the debug build (eff_debug_stubs.cu stands in)
_NOT_IN_DEBUG = ("eff_n192", "eff_n256", "eff_n512", "eff_batch")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# hidden visibility: only the C ABI (EFF_API in include/vmbd_eff.h) is exported,
# so that two builds loaded in one process (the library and its bounds-checked
# variant) share no symbol -- template statics such as the per-kernel shared
# memory attribute cache would otherwise be merged across them
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-Xcompiler",
         "-fvisibility=hidden"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources(debug: bool = False):
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    if debug:
        srcs = [p for p in srcs if not os.path.basename(p).startswith(_NOT_IN_DEBUG)]
    return srcs


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h")) + [os.path.abspath(__file__)]


def up_to_date(debug: bool = False) -> bool:
    lib = DEBUG_LIB if debug else LIB
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force: bool = False, verbose: bool = False, debug: bool = False) -> str:
    lib = DEBUG_LIB if debug else LIB
    if not force and up_to_date(debug):
        return lib
    nvcc = _nvcc()
    obj_dir = os.path.join(OUT_DIR, "obj_debug" if debug else "obj")
    os.makedirs(obj_dir, exist_ok=True)
    extra = ["-DEFF_DEBUG"] if debug else []

    def compile_one(src):
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    srcs = sources(debug)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


def build_all(force: bool = False) -> None:
    """The product library and its bounds-checked variant, compiled together."""
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(lambda d: build(force=force, debug=d), (False, True)))


if __name__ == "__main__":
    print(build(force=True, verbose=True))
