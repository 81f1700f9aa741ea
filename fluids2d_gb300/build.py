"""Build the CUDA library of fluids2d_gb300 in-tree.

Compiles ``csrc/*.cu`` for sm_103a with nvcc (one process per translation
unit, in parallel) and links ``_build/libfluids2d_gb300.so``. No cmake, no
torch extension machinery: the product is a plain C-ABI shared library
(``include/fluids2d_gb300.h``) loaded with ctypes.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libfluids2d_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["api.cu", "stage.cu", "mg.cu", "sweeps.cu", "mesh_host.cu",
           "noalloc.cu", "ensemble.cu", "solver.cu", "adjoint.cu", "nsolver.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-O2", "--expt-relaxed-constexpr", "-I", INCLUDE]


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if os.path.exists(cand):
            return cand
        raise RuntimeError("nvcc not found")
    return exe


def _deps():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
           if f.endswith((".cu", ".cuh", ".h"))]
    out.append(os.path.join(INCLUDE, "fluids2d_gb300.h"))
    return out


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [cc] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
