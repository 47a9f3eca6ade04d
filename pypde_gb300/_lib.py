"""ctypes binding of libpypde_gb300.so (the C ABI in include/pgx.h).

The library is mandatory: importing a compute function without it raises.
There is no CPU fallback anywhere in this package.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpypde_gb300.so")

MAX_ARR, MAX_MAT, MAX_LEN, MAX_PAR, MAX_OPS, MAX_SLOTS, LMAX = 24, 16, 16, 16, 96, 8, 2112

OP = dict(LOAD=1, LOAD_ADD=2, LOAD_MUL=3, STORE=4, STORE_ADD=5, SCALE=6, AXPY=7, MUL=8, COPY=9,
          SETLEN=10, STENCIL=11, STENCIL_T=12, TDMA2=13, DIFF=14, DCT=15, BANDED=17, DENSE=18,
          FDMA=19, POISSON=20, ZERO00=21, DIFF_T=22, FDMA_T=23, POISSON_T=24)
DCT_RAW, DCT_FWD, DCT_BWD, DCT_FWD_T, DCT_BWD_T = 0, 1, 2, 3, 4
CHAIN_WARP = 1  # op.k flag of the chain ops: one warp per chain (PGX_CHAIN_WARP)
DENSE_MMA = 2   # op.k flag of DENSE: contraction on the FP64 tensor cores (PGX_DENSE_MMA)
DCT_SLOT = 16   # op.k flag of DCT: the FFT in the slot's own lines and the spare (PGX_DCT_SLOT)
MAX_THREADS, MAX_THREADS_FFT = 1024, 768  # largest CTA; with DCT ops (PGX_MAX_THREADS[_FFT])


class PgxArray(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("s0", ctypes.c_int64), ("s1", ctypes.c_int64),
                ("n0", ctypes.c_int32), ("n1", ctypes.c_int32)]


class PgxInstance(ctypes.Structure):
    _fields_ = [("arr", PgxArray * MAX_ARR), ("mat", ctypes.c_void_p * MAX_MAT),
                ("len", ctypes.c_int32 * MAX_LEN), ("par", ctypes.c_double * MAX_PAR)]


class PgxOp(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int16), ("a", ctypes.c_int16), ("b", ctypes.c_int16),
                ("arr", ctypes.c_int16), ("mat", ctypes.c_int16), ("len", ctypes.c_int16),
                ("par", ctypes.c_int16), ("k", ctypes.c_int16), ("alpha", ctypes.c_double)]


class PgxProgram(ctypes.Structure):
    _fields_ = [("axis", ctypes.c_int32), ("lines_len", ctypes.c_int32), ("tb", ctypes.c_int32),
                ("lcap", ctypes.c_int32), ("nslots", ctypes.c_int32), ("nops", ctypes.c_int32),
                ("fft_n", ctypes.c_int32), ("nthreads", ctypes.c_int32), ("ops", PgxOp * MAX_OPS)]


assert ctypes.sizeof(PgxInstance) == 32 * MAX_ARR + 8 * MAX_MAT + 4 * MAX_LEN + 8 * MAX_PAR
assert ctypes.sizeof(PgxProgram) == 32 + 24 * MAX_OPS

_lib = None

SIGNATURES = {
    "pgx_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "pgx_last_cuda_error": (ctypes.c_int, []),
    "pgx_version": (ctypes.c_int, []),
    "pgx_program_smem": (ctypes.c_int64, [ctypes.c_void_p]),
    "pgx_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pgx_check_instance": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pgx_fp64_fma_probe": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_void_p]),
    "pgx_fp64_fma_probe_flops": (ctypes.c_int64, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "pgx_run_persistent": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                          ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                          ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_int64, ctypes.c_void_p]),
    "pgx_persistent_shape": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p]),
    "pgx_persist_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pgx_run_batched": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                       ctypes.c_void_p]),
    "pgx_dct1": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_cheb_transform_2d": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                             ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "pgx_cheb_transform_2d_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64,
                                                     ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_cheb_diff": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                     ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_cheb_diff_t": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                       ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_fdma_solve_t": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_poisson_solve_t": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                           ctypes.c_int32, ctypes.c_void_p]),
    "pgx_stencil_plan_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_stencil_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pgx_stencil_to_chebyshev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                                ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                                ctypes.c_int32, ctypes.c_void_p]),
    "pgx_stencil_from_chebyshev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                                  ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_stencil_transpose": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                             ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.c_void_p]),
    "pgx_stencil_from_chebyshev_t": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                                    ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                                    ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_tdma_plan_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                            ctypes.c_int32, ctypes.c_void_p]),
    "pgx_tdma_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pgx_tdma_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                      ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_void_p]),
    "pgx_fdma_plan_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int32, ctypes.c_void_p]),
    "pgx_twodma_plan_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_fdma_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pgx_fdma_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                      ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_poisson_plan_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                               ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_poisson_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pgx_poisson_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_int32, ctypes.c_void_p]),
    "pgx_matrix_plan_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "pgx_matrix_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pgx_matrix_plan_is_banded": (ctypes.c_int, [ctypes.c_void_p]),
    "pgx_matrix_apply": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_void_p]),
    "pgx_dct_table": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p]),
}


class PgxError(RuntimeError):
    pass


def lib():
    """Load (once) and return the ctypes handle; raise if the library is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PgxError("libpypde_gb300.so is not built: run `python -m pypde_gb300.build` "
                           "(pypde_gb300 has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc, what=""):
    if rc != 0:
        L = lib()
        msg = L.pgx_error_string(rc).decode()
        if rc == 2:
            msg += " (cudaError %d)" % L.pgx_last_cuda_error()
        raise PgxError("%s failed: %s" % (what or "pgx call", msg))


def f64(a):
    """Host float64 contiguous array + its ctypes pointer."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.c_void_p)


def op(code, a=0, b=-1, arr=-1, mat=-1, len=-1, k=0, alpha=1.0, par=-1):  # noqa: A002
    o = PgxOp()
    o.code, o.a, o.b, o.arr, o.mat, o.len, o.par, o.k, o.alpha = OP[code], a, b, arr, mat, len, par, k, alpha
    return o


def smem_bytes(prog):
    return lib().pgx_program_smem(ctypes.byref(prog))
