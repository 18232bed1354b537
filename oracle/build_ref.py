"""Build recipe for ``oracle/_ref``: the reference's hot-path kernels
(``gputools.cu``) compiled for the CPU.

TEST INFRASTRUCTURE ONLY.  Compiles ``ref_launch.cpp`` (which #includes the
reference's ``gputools.cu`` from where it lies, through a CUDA-execution-model
shim) with g++ into ``oracle/_ref/libref_gputools.so``.  Does nothing when the
reference checkout is absent (it exists only where fixtures are generated).

The checkout is the directory named by ``VMBD_REFERENCE_DIR``, else a
``reference`` directory beside this repository.

Usage: ``python oracle/build_ref.py [reference_dir]``.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_gputools.so")

def reference_dir() -> str:
    """Where the reference checkout lies: ``$VMBD_REFERENCE_DIR``, else
    ``../reference`` relative to the repository root."""
    env = os.environ.get("VMBD_REFERENCE_DIR")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


DEFAULT_REF = reference_dir()


def build(ref_dir: str = DEFAULT_REF, quiet: bool = False) -> str | None:
    src = os.path.join(ref_dir, "gputools.cu")
    if not os.path.exists(src):
        if not quiet:
            print(f"[oracle/_ref] {src} not present: skipped")
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    launch = os.path.join(HERE, "ref_launch.cpp")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src),
                                                            os.path.getmtime(launch)):
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-w",
           "-I", os.path.join(HERE, "ref_include"),
           f'-DREF_GPUTOOLS_CU="{src}"', launch, "-o", LIB]
    subprocess.run(cmd, check=True)
    if not quiet:
        print(f"[oracle/_ref] built {LIB}")
    return LIB


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF)
