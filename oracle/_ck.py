"""ctypes access to oracle/kernels.c (test infrastructure): the oracle's banded sweeps and derivative
recurrence compiled, the same operations as the NumPy restatement.  ``build()`` compiles it into
oracle/_build/; without the library the oracle keeps its NumPy loops."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "kernels.c")
LIB = os.path.join(HERE, "_build", "liboracle_kernels.so")
_lib = None


def build(force=False):
    """gcc -O2, no floating-point contraction (bit-equal to the NumPy loops); returns the path."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        tmp = "%s.%d.tmp" % (LIB, os.getpid())   # concurrent builders each write their own file
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, SRC], check=True)
        os.replace(tmp, LIB)
    return LIB


def lib():
    """The loaded library, or None when it is not built (a build older than kernels.c is rebuilt
    first, or left unused when that fails)."""
    global _lib
    if _lib is None and os.path.exists(LIB) and os.path.getmtime(LIB) < os.path.getmtime(SRC):
        try:
            build()
        except Exception:  # no compiler: the NumPy loops run
            return None
    if _lib is None and os.path.exists(LIB):
        L = ctypes.CDLL(LIB)
        P, I = ctypes.c_void_p, ctypes.c_int
        L.ok_fdma_lu.argtypes = [P, P, P, P, I, I]
        L.ok_fdma_solve.argtypes = [P, P, P, P, I, P, I, I]
        L.ok_twodma_solve.argtypes = [P, P, P, I, I]
        L.ok_tdma_offset.argtypes = [P, P, P, P, P, P, P, I, I, I]
        L.ok_cheb_diff1.argtypes = [P, P, I, I]
        _lib = L
    return _lib


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def c64(a):
    """C-contiguous float64 (a copy only when needed)."""
    return np.ascontiguousarray(a, dtype=np.float64)
