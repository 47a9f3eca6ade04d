"""Every launch the fused forward and reverse-mode steps build passes the C ABI's instance checks.

pgx_run_batched reads its instance descriptors from device memory and so cannot check them;
FusedBatch checks every member's host descriptor with pgx_check_instance when it builds a
launch (``_group_launch``).  Here the same construction runs on the CPU for batches of mixed sizes (Euler / RK3,
beta, both forms, both T bases, FFT and dense DCT, the forward and the reverse-mode passes) and
every tile candidate of every launch: the instance arrays and tables are stand-in host tensors
of the real shapes, and no kernel runs.
"""
import ctypes
import types

import numpy as np
import pytest
import torch

from pypde_gb300 import _lib
from pypde_gb300.host import pseudoinverse_d2, stencil_matrix
from pypde_gb300.navier import fused as F
from pypde_gb300.navier import fused_adjoint as FA
from pypde_gb300.templates import poisson2d_matrices

DCT_NAMES = ("dct", "dct_fwd", "dct_bwd", "dct_fwd_t", "dct_bwd_t")


def stand_in_instance(N, M, dealias, tk, rk3, beta):
    """The arrays, tables, lengths and stage maps of one instance, as _Instance and
    add_adjoint_buffers lay them out, on host tensors."""
    Nd, Md = (int(1.5 * N), int(1.5 * M)) if dealias else (N, M)
    z = lambda r, c: torch.zeros((r, c), dtype=torch.float64)  # noqa: E731
    ra, dt, scale, bt = 1e5, 0.01, (0.5, 0.5), (0.5 if beta else 1.0)
    nu = kappa = float(np.sqrt(1.0 / ra))
    I = types.SimpleNamespace(N=N, M=M, Nd=Nd, Md=Md, nstage=3 if rk3 else 1)
    a = {k: z(N - 2, M - 2) for k in ("UG", "VG", "TG", "PG")}
    a["PRES"] = z(N, M)
    a["TBCC"], a["DTB1"], a["DTB2"] = z(N, M), z(Nd, Md), z(N, M)
    a.update({k: z(*s) for k, s in F.scratch_shapes(N, M, Nd, Md, beta).items()})
    I.lens, I.par = F.instance_params(N, M, dealias, dt, nu, kappa, scale, beta=bt)

    def mats(n):
        return stencil_matrix("CN", n), pseudoinverse_d2(n)[2:, :], np.eye(n)[2:, :]

    fd = poisson2d_matrices(mats(N), mats(M), True, scale)
    host = {**F.global_tables_host(), **F.host_tables(N, M, tk, dt * bt, nu, kappa, scale, fd, adjoint=True)}
    I.tables = {k: torch.as_tensor(np.ascontiguousarray(v, dtype=np.float64)) for k, v in host.items()}
    I.stage_par, I.stage_tables, I.stage_arrays = [I.par], [{}], [{}]
    if rk3:
        for k in ("UX_A", "UX_B", "UZ_A", "UZ_B"):
            a[k] = z(Nd, Md)
        adi = {k: I.tables[k] for k in ("Ax_U", "Ax_T", "Ay_U", "Ay_T")}
        I.stage_par, I.stage_tables, I.stage_arrays = [I.par] * 3, [adi] * 3, []
        for st in range(3):
            cur, old = ("A", "A") if st == 0 else (("B", "A") if st == 1 else ("A", "B"))
            I.stage_arrays.append({"UXC": "UX_" + cur, "UZC": "UZ_" + cur, "UXO": "UX_" + old,
                                   "UZO": "UZ_" + old})
    # reverse mode (add_adjoint_buffers)
    for k in FA.BAR_STATE:
        a[k] = torch.zeros_like(a[k[1:]])
    a.update({k: z(*s) for k, s in FA.adjoint_shapes(N, M, Nd, Md, beta, rk3).items()})
    if rk3:
        I.stage_arrays = [dict(st, **carry) for st, carry in zip(I.stage_arrays, FA.RK3_CARRY)]
    I.arrays = a
    I.dct_x = I.dct_y = {k: 4096 for k in DCT_NAMES}   # device table addresses: any non-null value
    I.lines = lambda prog: I.lens[prog.lines] if prog.lines else 0
    I.fill = types.MethodType(F._Instance.fill, I)
    return I


def stand_in_batch(shapes, dealias, tk, fft, rk3, beta, split):
    fb = F.FusedBatch.__new__(F.FusedBatch)
    fb.insts = [stand_in_instance(N, M, dealias, tk, rk3, beta) for N, M in shapes]
    fb.fft, fb.nstage, fb.tkind, fb.split, fb.beta = fft, 3 if rk3 else 1, tk, split, beta
    return fb


def host_descriptors(d_insts):
    n = d_insts.numel() // ctypes.sizeof(_lib.PgxInstance)
    return (_lib.PgxInstance * n).from_buffer_copy(d_insts.numpy().tobytes())


def check_every_tile(fb, progs):
    lib = _lib.lib()
    checked = 0
    for prog in progs:
        nv = len(prog.variants)
        for st in range(fb.nstage):
            d = fb._d_insts(prog, st)
            host = host_descriptors(d)
            for key, members in fb._groups(prog):
                lines = [fb.insts[k].lines(prog) for k in members]
                for tile in F._candidates(prog, sum(lines) * nv, key[0], key[1], max(lines)):
                    tb, nt, wc, sd, dm = tile
                    L = fb._group_launch(prog, d, key, members, tb, nt, wc, prog.name, sd, dm)
                    for k in members:
                        for v in range(nv):
                            rc = lib.pgx_check_instance(ctypes.byref(L["P"]), ctypes.byref(host[k * nv + v]))
                            assert rc == 0, (prog.name, st, key, tile, k, v, rc)
                            checked += 1
    return checked


@pytest.fixture(autouse=True)
def host_device(monkeypatch):
    monkeypatch.setattr(F, "device", lambda: torch.device("cpu"))
    monkeypatch.setattr(FA, "device", lambda: torch.device("cpu"))


SHAPES = [(33, 33), (65, 33), (17, 65), (129, 129)]


@pytest.mark.parametrize("tk", ["CD", "CN"])
@pytest.mark.parametrize("rk3", [False, True], ids=["euler", "rk3"])
@pytest.mark.parametrize("beta", [False, True], ids=["b1", "beta"])
@pytest.mark.parametrize("split", [False, True], ids=["fused", "per-field"])
def test_launch_descriptors_pass_the_instance_checks(tk, rk3, beta, split):
    fb = stand_in_batch(SHAPES, True, tk, True, rk3, beta, split)
    progs = F.build_programs(tk, True, rk3=rk3, split=split, beta=beta)
    aprogs = FA.build_adjoint_programs(tk, True, split, beta, rk3=rk3)
    assert check_every_tile(fb, progs + aprogs) > 0


@pytest.mark.parametrize("dealias", [True, False])
def test_launch_descriptors_dense_dct_and_large(dealias):
    fb = stand_in_batch([(33, 17), (40, 24)], dealias, "CD", False, False, False, False)
    assert check_every_tile(fb, F.build_programs("CD", False) + FA.build_adjoint_programs("CD", False)) > 0
    fb = stand_in_batch([(513, 257)], dealias, "CD", True, False, False, None)
    assert check_every_tile(fb, F.build_programs("CD", True, split=True)) > 0


@pytest.mark.parametrize("shapes", [[(9, 7), (12, 13)], [(19, 33), (40, 24)], [(257, 129)], [(65, 513)]],
                         ids=["tiny", "odd", "257x129", "65x513"])
@pytest.mark.parametrize("rk3", [False, True], ids=["euler", "rk3"])
def test_launch_descriptors_other_shapes(shapes, rk3):
    for split in (False, True):
        for dealias in (True, False):
            fb = stand_in_batch(shapes, dealias, "CN", True, rk3, False, split)
            progs = F.build_programs("CN", True, rk3=rk3, split=split)
            assert check_every_tile(fb, progs + FA.build_adjoint_programs("CN", True, split, rk3=rk3)) > 0


def test_launch_without_host_descriptors_is_refused():
    """Descriptors not made by _d_insts carry no host copy: building a launch over them raises
    instead of skipping the instance checks."""
    fb = stand_in_batch([(33, 33)], True, "CD", True, False, False, False)
    prog = F.build_programs("CD", True)[0]
    d = fb._d_insts(prog, 0)
    bare = d.clone()  # same bytes, no host copy attached
    (key, members), = fb._groups(prog)
    tb, nt, wc, sd, dm = F._pick(prog, fb.insts[0].lines(prog), key[0], key[1], fb.insts[0].lines(prog))
    fb._group_launch(prog, d, key, members, tb, nt, wc, prog.name, sd, dm)
    with pytest.raises(RuntimeError, match="host copy"):
        fb._group_launch(prog, bare, key, members, tb, nt, wc, prog.name, sd, dm)
