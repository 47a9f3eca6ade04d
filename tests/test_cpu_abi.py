"""CPU checks of the product side: the C-ABI library builds, loads and exports every
entry point include/pgx.h declares; ctypes mirrors match the C layouts; host-side
setup matrices match the oracle.  No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, rel_err


def declared_functions():
    src = open(os.path.join(ROOT, "include", "pgx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pgx_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from pypde_gb300 import build
    lib = ctypes.CDLL(build.build())
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header():
    from pypde_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_struct_layouts():
    from pypde_gb300 import _lib
    assert ctypes.sizeof(_lib.PgxArray) == 32
    assert ctypes.sizeof(_lib.PgxOp) == 24
    assert ctypes.sizeof(_lib.PgxInstance) == 32 * 24 + 8 * 16 + 4 * 16 + 8 * 16
    assert ctypes.sizeof(_lib.PgxProgram) == 32 + 24 * 96


def test_library_calls_without_gpu_are_safe():
    from pypde_gb300 import _lib
    L = _lib.lib()
    assert L.pgx_version() == 1
    assert L.pgx_error_string(1).startswith(b"invalid argument")
    assert L.pgx_dct1(None, 1, 1, 5, None, 1, 1, 5, 5, 1, 0, 0, None) == 1


@pytest.mark.parametrize("N", [17, 33, 65])
def test_host_matrices_match_oracle(N):
    from oracle import spectral as sp
    from oracle import linalg as ol
    from pypde_gb300 import host
    assert np.array_equal(host.gauss_lobatto(N - 1), sp.gauss_lobatto(N - 1))
    for key in ("CD", "CN", "DC", "NC"):
        assert np.array_equal(host.stencil_matrix(key, N), sp.stencil(key, N))
    assert rel_err(host.pseudoinverse_d2(N), sp.pseudoinverse_d2(N)) < 1e-15
    A = sp.B2(N) @ sp.stencil("CD", N) - 0.01 * sp.I2(N) @ sp.stencil("CD", N)
    for a, b in zip(host.fdma_lu(A), ol.fdma_factor(A)):
        assert rel_err(a, b) < 1e-15


@pytest.mark.parametrize("tkind", ["CD", "CN"])
@pytest.mark.parametrize("fft", [True, False])
def test_fused_programs_fit_the_abi(tkind, fft):
    """Every fused pass (Euler and RK3-stage variants) respects the C-ABI limits and uses only
    slots it declares."""
    from pypde_gb300 import _lib
    from pypde_gb300.navier.fused import build_programs
    progs = []
    for beta in (False, True):
        progs += (build_programs(tkind, fft, beta=beta) + build_programs(tkind, fft, rk3=True, beta=beta) +
                  build_programs(tkind, fft, split=True, beta=beta) +
                  build_programs(tkind, fft, rk3=True, split=True, beta=beta))
    assert len(progs) == (11 + 11 + 12 + 12) + (12 + 12 + 13 + 13)
    uses_b = {_lib.OP[k] for k in ("AXPY", "MUL", "COPY")}
    for p in progs:
        assert len(p.ops) <= _lib.MAX_OPS, p.name
        assert len(p.arrs) <= _lib.MAX_ARR, p.name
        assert len(p.mats) <= _lib.MAX_MAT, p.name
        assert 1 <= p.nslots <= _lib.MAX_SLOTS
        chain = {_lib.OP[k] for k in ("DIFF", "TDMA2", "FDMA")}
        for o in p.ops:
            assert 0 <= o.a < p.nslots, p.name
            if o.code in uses_b:
                assert 0 <= o.b < p.nslots, p.name
            if o.code in chain:
                assert o.a + max(o.b, 1) <= p.nslots, p.name
            if o.code == _lib.OP["FDMA"]:
                assert o.mat + max(o.b, 1) <= len(p.mats)
            assert o.len < _lib.MAX_LEN and o.par < _lib.MAX_PAR
        # every array stored is either state or scratch; every loaded array is defined
        assert p.axis in (0, 1)


def test_program_checks_reject_malformed_dct_ops():
    """pgx_run refuses, before any launch, programs whose DCT ops could not run: no FFT buffers
    (fft_n < 2), more slots than the program has, or a CTA above the FFT build's 768 threads."""
    from pypde_gb300 import _lib
    L = _lib.lib()

    def prog(fft_n=9, nthreads=256, b=1, nslots=1):
        P = _lib.PgxProgram()
        P.axis, P.lines_len, P.tb, P.lcap, P.nslots, P.fft_n, P.nthreads = 0, 1, 2, 11, nslots, fft_n, nthreads
        ops = [_lib.op("LOAD", a=0, arr=0, len=0), _lib.op("DCT", a=0, b=b, mat=0, k=_lib.DCT_FWD),
               _lib.op("STORE", a=0, arr=1)]
        P.nops = len(ops)
        for i, o in enumerate(ops):
            P.ops[i] = o
        return P

    inst = _lib.PgxInstance()
    for P in (prog(fft_n=0), prog(fft_n=1), prog(nthreads=1024), prog(b=2, nslots=1)):
        assert L.pgx_run(ctypes.byref(P), ctypes.byref(inst), None) == 1   # PGX_E_ARG
    assert _lib.MAX_THREADS == 1024 and _lib.MAX_THREADS_FFT == 768


def test_in_slot_dct_flag():
    """PGX_DCT_SLOT (the FFT of a one-slot DCT op in the slot's own lines and the spare slot):
    pgx_program_smem drops the FFT buffers when every DCT op has it, pgx_run refuses it on a
    multi-slot op or an odd tile, and the host's length rule (dct_in_slot_ok) holds exactly for the
    even lengths whose radix plan (3s, then 4s, then one 2) has, or can be given by splitting a
    radix-4 stage or merging two radix-2 stages, an odd number of stages."""
    from pypde_gb300 import _lib
    from pypde_gb300.navier.fused import dct_in_slot_ok
    L = _lib.lib()

    def prog(k, b=1, tb=4):
        P = _lib.PgxProgram()
        P.axis, P.lines_len, P.tb, P.lcap, P.nslots, P.fft_n, P.nthreads = 0, 1, tb, 195, 2, 193, 128
        ops = [_lib.op("LOAD", a=0, arr=0, len=0), _lib.op("DCT", a=0, b=b, mat=0, k=k), _lib.op("STORE", a=0, arr=1)]
        P.nops = len(ops)
        for i, o in enumerate(ops):
            P.ops[i] = o
        return P

    plain = L.pgx_program_smem(ctypes.byref(prog(_lib.DCT_FWD)))
    slot = L.pgx_program_smem(ctypes.byref(prog(_lib.DCT_FWD | _lib.DCT_SLOT)))
    # 3 slot buffers of 4 x 195, the y_1 scalars (4 + 1); without the flag one FFT buffer of 2 pairs
    # x 192 complex values (the second is the spare slot)
    assert slot == 8 * (3 * 4 * 195 + 5) and plain == slot + 8 * 2 * 2 * 192
    inst = _lib.PgxInstance()
    for P in (prog(_lib.DCT_FWD | _lib.DCT_SLOT, b=2), prog(_lib.DCT_FWD | _lib.DCT_SLOT, tb=3)):
        assert L.pgx_run(ctypes.byref(P), ctypes.byref(inst), None) == 1   # PGX_E_ARG

    def odd_plan_exists(n):
        N = n - 1
        if N < 2 or N % 2:
            return False
        m, n3, n4, n2 = N, 0, 0, 0
        while m % 3 == 0:
            m, n3 = m // 3, n3 + 1
        while m % 4 == 0:
            m, n4 = m // 4, n4 + 1
        if m % 2 == 0:
            m, n2 = m // 2, n2 + 1
        if m != 1:
            return False
        return (n3 + n4 + n2) % 2 == 1 or n4 > 0 or n2 >= 2

    assert all(dct_in_slot_ok(n) == odd_plan_exists(n) for n in range(2, _lib.LMAX))
    assert [n for n in (7, 9, 17, 33, 49, 55, 97, 193) if dct_in_slot_ok(n)] == [9, 17, 33, 49, 97, 193]


def test_instance_checks_on_host_descriptors():
    """pgx_check_instance (no device needed) accepts a consistent descriptor and refuses one whose
    array is longer than the slot capacity, whose length exceeds it, or whose table is missing."""
    from pypde_gb300 import _lib
    L = _lib.lib()
    P = _lib.PgxProgram()
    P.axis, P.lines_len, P.tb, P.lcap, P.nslots, P.fft_n, P.nthreads = 0, 1, 2, 11, 1, 9, 256
    ops = [_lib.op("LOAD", a=0, arr=0, len=0), _lib.op("DCT", a=0, b=1, mat=0, k=_lib.DCT_FWD),
           _lib.op("STORE", a=0, arr=1)]
    P.nops = len(ops)
    for i, o in enumerate(ops):
        P.ops[i] = o

    def inst(n0=9, length=9, table=4096):
        I = _lib.PgxInstance()
        for a in (0, 1):
            I.arr[a].ptr, I.arr[a].s0, I.arr[a].s1, I.arr[a].n0, I.arr[a].n1 = 4096, 5, 1, n0, 5
        I.len[0], I.len[1] = length, 5
        I.mat[0] = table
        return I

    ok = inst()
    assert L.pgx_check_instance(ctypes.byref(P), ctypes.byref(ok)) == 0
    for bad in (inst(n0=12), inst(length=11), inst(table=0)):
        assert L.pgx_check_instance(ctypes.byref(P), ctypes.byref(bad)) == 1     # PGX_E_ARG
    assert L.pgx_check_instance(None, ctypes.byref(ok)) == 1


@pytest.mark.parametrize("shape", [(33, 33), (65, 129), (129, 129), (513, 257), (1025, 65)])
def test_tile_candidates_fit_the_launch_limits(shape):
    """Every tile the autotuner may try (and the default pick), for every forward / reverse-mode
    program form, fits the batched launch's shared memory (program + instance descriptor, the
    check pgx_run_batched makes) and the thread limit of the kernel build it runs on."""
    import ctypes
    from pypde_gb300 import _lib
    from pypde_gb300.navier.fused import (L_ND, _candidates, _pick, build_programs, instance_params, launch_program,
                                          program_maxlen)
    from pypde_gb300.navier.fused_adjoint import build_adjoint_programs
    N, M = shape
    lens, _ = instance_params(N, M, True, 0.01, 1e-3, 1e-3, (0.5, 0.5))
    progs = (build_programs("CD", True) + build_programs("CN", True, rk3=True, split=True, beta=True) +
             build_adjoint_programs("CD", True) + build_adjoint_programs("CN", True, split=True, beta=True, rk3=True))
    limit = 227 * 1024
    desc = -(-ctypes.sizeof(_lib.PgxInstance) // 16) * 16
    for prog in progs:
        lcap = (program_maxlen(prog, lens) + 1) | 1
        fft_n = lens[L_ND + prog.axis] if prog.has_dct else 0
        lines = lens[prog.lines]
        tiles = _candidates(prog, lines * len(prog.variants), lcap, fft_n, lines)
        tiles.append(_pick(prog, lines * len(prog.variants), lcap, fft_n, lines))
        for tb, nt, wc, sd, dm in tiles:
            P = launch_program(prog, (lcap, fft_n), tb, nt, wc, sd, dm)
            smem = _lib.smem_bytes(P)
            assert smem + desc + 1024 <= limit, (prog.name, shape, tb, nt, sd, dm, smem)
            has_dct = any(P.ops[i].code == _lib.OP["DCT"] for i in range(P.nops))
            assert nt % 32 == 0 and nt <= (_lib.MAX_THREADS_FFT if has_dct else _lib.MAX_THREADS), (prog.name, nt)
