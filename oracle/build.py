"""ORACLE - test infrastructure only: build recipe for the C restatement.

Compiles ``sweeps.c`` into ``oracle/_build/liboracle.so`` with gcc. The flags
keep the reference's arithmetic: ``-ffp-contract=off`` (no fused multiply-add,
like numba without fastmath and like Python floats) and ``-fno-builtin-pow``
(so that the ``_py`` entry points really call libm ``pow``, as Python's
``x**2`` does, instead of being folded to ``x*x``). OpenMP threads the sweeps
the way the reference's numba ``prange`` split does.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")


def build(force=False, verbose=False):
    src = [os.path.join(HERE, "sweeps.c")]
    deps = src + [os.path.join(HERE, "sweeps_body.h")]
    if (not force and os.path.exists(LIB) and
            all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps)):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-builtin-pow", "-o", tmp] + src + ["-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
