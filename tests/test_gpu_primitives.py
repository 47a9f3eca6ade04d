"""GPU parity of every reference-facing kernel against the oracle and the golden vectors.

Tolerance (stated by the parity target of the path): 1e-10 relative per
transform or solve, measured as max|gpu - ref| / max|ref|.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def pg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    import pypde_gb300
    return pypde_gb300


def host(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("N", [33, 40, 65])
def test_chebyshev_golden(pg, golden, N):
    CH = pg.Base(N, "CH")
    assert rel_err(host(CH.forward_fft(golden[f"ch{N}_f"])), golden[f"ch{N}_fwd"]) < TOL
    assert rel_err(host(CH.backward_fft(golden[f"ch{N}_c"])), golden[f"ch{N}_bwd"]) < TOL
    assert rel_err(host(CH.derivative(golden[f"ch{N}_c"], 1)), golden[f"ch{N}_d1"]) < TOL
    assert rel_err(host(CH.derivative(golden[f"ch{N}_c"], 2)), golden[f"ch{N}_d2"]) < TOL


@pytest.mark.parametrize("N", [33, 40, 65])
@pytest.mark.parametrize("key", ["CD", "CN"])
def test_galerkin_golden(pg, golden, N, key):
    B = pg.Base(N, key)
    f, c, v = golden[f"ch{N}_f"], golden[f"ch{N}_c"], golden[f"{key}{N}_v"]
    assert rel_err(host(B.forward_fft(f)), golden[f"{key}{N}_fwd"]) < TOL
    assert rel_err(host(B.backward_fft(v)), golden[f"{key}{N}_bwd"]) < TOL
    assert rel_err(host(B.to_chebyshev(v)), golden[f"{key}{N}_toch"]) < TOL
    assert rel_err(host(B.from_chebyshev(c)), golden[f"{key}{N}_fromch"]) < TOL
    assert rel_err(host(B.derivative(v, 1)), golden[f"{key}{N}_d1"]) < TOL
    assert rel_err(host(B.derivative(v, 2)), golden[f"{key}{N}_d2"]) < TOL


@pytest.mark.parametrize("n", [33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 17, 50, 28, 5, 3])
@pytest.mark.parametrize("axis", [0, 1])
def test_dct_sizes_vs_oracle(pg, n, axis):
    """Microbench sizes (N = 33..1025, seed 1) and their 3/2-dealiased lengths, both axes;
    forward/backward DCT against the oracle and the round trip."""
    from oracle import spectral as sp
    import torch
    rng = np.random.default_rng(1)
    f = rng.uniform(-1, 1, (n, 37) if axis == 0 else (37, n))
    ft = torch.as_tensor(f, device="cuda")
    CH = pg.Base(n, "CH")
    view = ft if axis == 0 else ft.T
    c = CH.forward_fft(view)
    ref_c = sp.cheb_forward(f, axis)
    assert rel_err(host(c if axis == 0 else c.T), ref_c) < TOL
    back = CH.backward_fft(c)
    assert rel_err(host(back if axis == 0 else back.T), f) < TOL
    raw = CH.dctn(view)
    assert rel_err(host(raw if axis == 0 else raw.T), sp.dct1(f, axis)) < TOL


@pytest.mark.parametrize("keys", [("CD", "CN"), ("CD", "CD"), ("CH", "CH")])
def test_field_2d_golden(pg, golden, keys):
    tag = "".join(keys)
    g = lambda k: golden[f"f2_{tag}_{k}"]  # noqa: E731
    fld = pg.Field([pg.Base(33, keys[0], dealias=3 / 2), pg.Base(20, keys[1], dealias=3 / 2)])
    assert rel_err(host(fld.forward(g("v"))), g("fwd")) < TOL
    assert rel_err(host(fld.backward(g("vh"))), g("bwd")) < TOL
    assert rel_err(host(fld.dealias.backward(g("vh"))), g("dbwd")) < TOL
    assert rel_err(host(fld.dealias.forward(g("vd"))), g("dfwd")) < TOL
    fld.vhat = g("vh")
    for d in ((1, 0), (0, 1), (2, 0), (0, 2), (1, 1)):
        assert rel_err(host(pg.grad(fld, d, scale=(0.5, 0.25))), g(f"grad{d[0]}{d[1]}")) < TOL
    assert rel_err(host(pg.galerkin_to_cheby(g("vh"), fld)), g("g2c")) < TOL
    assert rel_err(host(pg.cheby_to_galerkin(g("ch"), fld)), g("c2g")) < TOL


@pytest.mark.parametrize("dealias", [True, False])
def test_convective_term_golden(pg, golden, dealias):
    t = f"conv{int(dealias)}"
    fld = pg.Field([pg.Base(33, "CD", dealias=3 / 2), pg.Base(20, "CD", dealias=3 / 2)])
    dfld = pg.Field([pg.Base(33, "CH", dealias=3 / 2), pg.Base(20, "CH", dealias=3 / 2)])
    fld.vhat = golden[t + "_vh"]
    out = pg.convective_term(fld, golden[t + "_ux"], golden[t + "_uz"], deriv_field=dfld,
                             add_bc=golden[t + "_bc"], dealias=dealias, scale=(0.5, 0.5))
    assert rel_err(host(out), golden[t + "_out"]) < TOL


@pytest.mark.parametrize("keys", [("CD", "CD"), ("CN", "CD")])
def test_hholtz_adi_golden(pg, golden, keys):
    tag = "".join(keys)
    fld = pg.Field([pg.Base(33, keys[0]), pg.Base(25, keys[1])])
    sol = pg.solverplan_hholtz2d_adi(fld.xs, lam=0.01, scale=(0.5, 0.5))
    r = sol.solve_rhs(golden[f"hh_{tag}_b"])
    assert rel_err(host(r), golden[f"hh_{tag}_rhs"]) < TOL
    r = r + sol.solve_old(golden[f"hh_{tag}_old"])
    assert rel_err(host(r), golden[f"hh_{tag}_rhsold"]) < TOL
    assert rel_err(host(sol.solve_lhs(r)), golden[f"hh_{tag}_x"]) < TOL


@pytest.mark.parametrize("keys,singular", [(("CN", "CN"), True), (("CD", "CD"), False), (("CD", "CN"), False)])
def test_poisson_golden(pg, golden, keys, singular):
    tag = "".join(keys)
    fld = pg.Field([pg.Base(33, keys[0]), pg.Base(25, keys[1])])
    sol = pg.solverplan_poisson2d(fld.xs, singular=singular, scale=(0.5, 0.5))
    x = sol.solve_lhs(sol.solve_rhs(golden[f"po_{tag}_b"]))
    if singular:
        x[0, 0] = 0
    assert rel_err(host(x), golden[f"po_{tag}_x"]) < TOL


def test_banded_plans_vs_dense(pg):
    """test_methods.py:39-103 pattern: FDMA / TwoDMA plans along both axes vs np.linalg.solve."""
    import torch
    rng = np.random.default_rng(5)
    N, M = 20, 10
    l, d, u1, u2 = rng.random(N - 2), rng.random(N) + 4, rng.random(N - 2), rng.random(N - 4)
    A = np.diag(d) + np.diag(u1, 2) + np.diag(u2, 4) + np.diag(l, -2)
    b = rng.random((N, M))
    x = pg.PlanLHS(A, ndim=2, axis=0, method="fdma").solve(torch.as_tensor(b.copy(), device="cuda"))
    assert rel_err(host(x), np.linalg.solve(A, b)) < 1e-13
    x = pg.PlanLHS(A, ndim=2, axis=1, method="fdma").solve(torch.as_tensor(b.T.copy(), device="cuda"))
    assert rel_err(host(x), np.linalg.solve(A, b).T) < 1e-13
    x = pg.PlanLHS(A, ndim=1, axis=0, method="fdma").solve(torch.as_tensor(b[:, 0].copy(), device="cuda"))
    assert rel_err(host(x), np.linalg.solve(A, b[:, 0])) < 1e-13
    dd, uu = rng.random(N) + 2, rng.random(N - 2)
    A2 = np.diag(dd) + np.diag(uu, 2)
    x = pg.PlanLHS(A2, ndim=2, axis=0, method="twodma").solve(torch.as_tensor(b.copy(), device="cuda"))
    assert rel_err(host(x), np.linalg.solve(A2, b)) < 1e-13
    x = pg.PlanLHS(A2, ndim=2, axis=1, method="twodma").solve(torch.as_tensor(b.T.copy(), device="cuda"))
    assert rel_err(host(x), np.linalg.solve(A2, b).T) < 1e-13
    R = rng.random((N, N))
    x = pg.SolverPlan()
    x.add_rhs(pg.PlanRHS(R, ndim=2, axis=1))
    x.add_lhs(pg.PlanLHS(A, ndim=2, axis=1, method="numpy"))
    bb = rng.random((M, N))
    out = x.solve_lhs(x.solve_rhs(torch.as_tensor(bb, device="cuda")))
    assert rel_err(host(out), np.linalg.solve(A, (bb @ R.T).T).T) < 1e-12


def test_tdma_plan_offset2(pg):
    import ctypes
    import torch
    from pypde_gb300 import _lib
    rng = np.random.default_rng(6)
    n, m = 30, 7
    a, b, c = rng.random(n - 2), rng.random(n) + 3, rng.random(n - 2)
    T = np.diag(a, -2) + np.diag(b) + np.diag(c, 2)
    d = rng.random((n, m))
    h = ctypes.c_void_p()
    ptr = lambda v: v.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    _lib.check(_lib.lib().pgx_tdma_plan_create(ptr(a), ptr(b), ptr(c), n, 2, ctypes.byref(h)))
    dt = torch.as_tensor(d, device="cuda")
    x = torch.empty_like(dt)
    _lib.check(_lib.lib().pgx_tdma_solve(h, dt.data_ptr(), m, 1, x.data_ptr(), m, 1, m, 0,
                                         torch.cuda.current_stream().cuda_stream))
    assert rel_err(host(x), np.linalg.solve(T, d)) < 1e-13
    assert _lib.lib().pgx_tdma_plan_create(ptr(a), ptr(b), ptr(c), n, 1, ctypes.byref(h)) == 1  # k != 2 rejected
    _lib.lib().pgx_tdma_plan_destroy(h)


def test_c_abi_rejects_bad_arguments(pg):
    from pypde_gb300 import _lib
    L = _lib.lib()
    assert L.pgx_dct1(None, 1, 1, 5, None, 1, 1, 5, 5, 1, 0, 0, None) == 1
    assert L.pgx_dct1(1, 1, 1, 9, 1, 1, 1, 5, 5, 1, 0, 0, None) == 1  # n_in > n
    assert L.pgx_dct1(1, 1, 1, 5, 1, 1, 1, 5, 5, 1, 2, 0, None) == 1  # axis 2
    assert L.pgx_fdma_solve(None, 1, 1, 1, 1, 0, None) == 4  # null plan
    assert L.pgx_cheb_diff(1, 1, 1, 1, 1, 1, 2, 1, 0, 1, None) == 1  # n < 3
    # the transposed (reverse-mode) entry points check the same way
    assert L.pgx_dct1(1, 1, 1, 5, 1, 1, 1, 5, 5, 1, 0, 5, None) == 1  # no mode 5
    assert L.pgx_cheb_diff_t(1, 1, 1, 1, 1, 1, 2, 1, 0, 1, None) == 1  # n < 3
    assert L.pgx_fdma_solve_t(None, 1, 1, 1, 1, 0, None) == 4  # null plan
    assert L.pgx_poisson_solve_t(None, 1, 1, 1, 0, None) == 4
    assert L.pgx_stencil_transpose(None, 1, 1, 1, 1, 1, 1, 1, 0, None) == 4
    assert L.pgx_stencil_from_chebyshev_t(None, 1, 1, 1, 1, 1, 1, 1, 0, None) == 4


RBC = [
    ("rbc_lin33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 10, 0, 1e-2),
    ("rbc_lin33nd", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=False, integrator="eu"), 10, 0, 1e-2),
    ("rbc_lin33x17", "linear", (33, 17), dict(ra=3e4, dt=0.01, dealias=True, integrator="eu", aspect=2.0), 10, 5, 1e-2),
    ("rbc_rbc33", "rbc", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 10, 1, 1e-2),
    ("rbc_zero33", "zero", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 10, 2, 1e-2),
    ("rbc_rk3_33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="rk3"), 5, 3, 1e-2),
    ("rbc_beta33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu", beta=0.5), 5, 4, 1e-2),
]


@pytest.mark.parametrize("fused", [False, None], ids=["plain", "default"])
@pytest.mark.parametrize("case", RBC, ids=[c[0] for c in RBC])
def test_rbc2d_plain_golden(pg, golden, case, fused):
    """update(fused=False): the operation-by-operation path; update(): the default (fused) step."""
    from pypde_gb300.navier.rbc2d import NavierStokes
    tag, kind, shape, cfg, nsteps, seed, amp = case
    ns = NavierStokes(case=kind, shape=shape, pr=1.0, tsave=None, **cfg)
    ns.set_temperature_noise(seed, amp)
    assert rel_err(host(ns.T.vhat), golden[tag + "_T0"]) < TOL
    ns.update(fused=fused)
    assert (ns._fused is None) == (fused is False)
    st = ns.state()
    for name in ("T", "U", "V", "P", "pres"):
        assert rel_err(st[name], golden[f"{tag}_s1_{name}"]) < 1e-9, name
    for _ in range(nsteps - 1):
        ns.update(fused=fused)
    st = ns.state()
    for name in ("T", "U", "V", "P", "pres"):
        assert rel_err(st[name], golden[f"{tag}_s{nsteps}_{name}"]) < 1e-8, name
    nu, nuv, ke = golden[f"{tag}_s{nsteps}_scalars"]
    Nu, Nuv = ns.eval_Nu()
    assert abs(Nu - nu) / abs(nu) < 1e-8
    assert abs(Nuv - nuv) / abs(nuv) < 1e-8
    assert abs(ns.eval_KE() - ke) / abs(ke) < 1e-8


@pytest.mark.parametrize("shape", [(33, 20), (65, 129)])
def test_cheb_transform_2d_dealiased(pg, shape):
    """pgx_cheb_transform_2d = deriv_field.dealias.backward / .forward (field.py:14-56) for CH x CH."""
    import torch
    from pypde_gb300 import _lib
    from oracle import field as ofo
    N, M = shape
    Nd, Md = int(1.5 * N), int(1.5 * M)
    sp2 = ofo.Space2D(("CH", "CH"), (N, M))
    rng = np.random.default_rng(8)
    c = rng.uniform(-1, 1, (N, M))
    v = rng.uniform(-1, 1, (Nd, Md))
    L = _lib.lib()
    st = torch.cuda.current_stream().cuda_stream
    ct = torch.as_tensor(c, device="cuda")
    out = torch.empty((Nd, Md), dtype=torch.float64, device="cuda")
    work = torch.empty(Nd * M, dtype=torch.float64, device="cuda")
    _lib.check(L.pgx_cheb_transform_2d(ct.data_ptr(), M, 1, N, M, out.data_ptr(), Md, 1, Nd, Md, Nd, Md,
                                       _lib.DCT_BWD, work.data_ptr(), work.numel(), st))
    assert rel_err(host(out), sp2.dealias_backward(c)) < TOL
    vt = torch.as_tensor(v, device="cuda")
    out2 = torch.empty((N, M), dtype=torch.float64, device="cuda")
    work2 = torch.empty(N * Md, dtype=torch.float64, device="cuda")
    _lib.check(L.pgx_cheb_transform_2d(vt.data_ptr(), Md, 1, Nd, Md, out2.data_ptr(), M, 1, N, M, Nd, Md,
                                       _lib.DCT_FWD, work2.data_ptr(), work2.numel(), st))
    assert rel_err(host(out2), sp2.dealias_forward(v)) < TOL
    assert L.pgx_cheb_transform_2d(ct.data_ptr(), M, 1, N, M, out.data_ptr(), Md, 1, Nd, Md, Nd, Md,
                                   _lib.DCT_BWD, work.data_ptr(), Nd * M - 1, st) == 1  # workspace too small


def _dct_line_program(n, nlines, tb, nthreads, flags):
    """LOAD -> forward DCT-I of n points -> STORE over ``nlines`` contiguous lines, through pgx_run
    (the C ABI), with ``flags`` added to the DCT op's k; returns (input, output) on the host."""
    import ctypes
    import torch
    from pypde_gb300 import _lib
    L = _lib.lib()
    x = torch.as_tensor(np.random.default_rng(n).uniform(-1, 1, (nlines, n)), device="cuda")
    y = torch.full_like(x, 7.0)
    tab = ctypes.c_void_p()
    _lib.check(L.pgx_dct_table(n, ctypes.byref(tab)), "dct table")
    P = _lib.PgxProgram()
    P.axis, P.lines_len, P.tb, P.lcap, P.nslots, P.fft_n, P.nthreads = 1, 1, tb, (n + 1) | 1, 1, n, nthreads
    ops = [_lib.op("LOAD", a=0, arr=0, len=0), _lib.op("DCT", a=0, b=1, mat=0, k=_lib.DCT_FWD | flags),
           _lib.op("STORE", a=0, arr=1)]
    P.nops = len(ops)
    for i, o in enumerate(ops):
        P.ops[i] = o
    inst = _lib.PgxInstance()
    for a, t in ((0, x), (1, y)):
        inst.arr[a].ptr, inst.arr[a].s0, inst.arr[a].s1, inst.arr[a].n0, inst.arr[a].n1 = t.data_ptr(), n, 1, nlines, n
    inst.len[0], inst.len[1] = n, nlines
    inst.mat[0] = tab.value
    _lib.check(L.pgx_run(ctypes.byref(P), ctypes.byref(inst), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
               "pgx_run")
    torch.cuda.synchronize()
    return host(x), host(y)


@pytest.mark.parametrize("tb,nthreads", [(2, 64), (4, 32)])    # CTA-wide form, warp-local form
@pytest.mark.parametrize("n", [9, 13, 17, 19, 33, 49, 97, 129])
def test_in_slot_dct_matches_buffered_and_oracle(pg, n, tb, nthreads):
    """PGX_DCT_SLOT (the FFT in the slot's own lines and the spare slot, the stage count made odd:
    8 -> 2,2,2; 12 -> 3,2,2; 16 -> 4,2,2; 96 -> 3,4,2,2,2; 128 -> 4,4,2,2,2 points; 18, 32, 48 keep
    theirs) gives the buffered transform to rounding and the oracle's forward Chebyshev transform."""
    from oracle import spectral as sp
    x, got = _dct_line_program(n, 6, tb, nthreads, _lib_flag("DCT_SLOT"))
    _, ref = _dct_line_program(n, 6, tb, nthreads, 0)
    assert rel_err(got, ref) < 1e-13
    assert rel_err(got, sp.cheb_forward(x, axis=1)) < TOL


@pytest.mark.parametrize("n", [7, 55])
def test_in_slot_dct_refuses_lengths_without_an_odd_plan(pg, n):
    """n - 1 = 2 * 3^b with b odd has no FFT plan with an odd number of stages: the in-slot transform
    refuses (NaN outputs, no fault), the buffered one transforms."""
    _, got = _dct_line_program(n, 6, 2, 64, _lib_flag("DCT_SLOT"))
    _, ref = _dct_line_program(n, 6, 2, 64, 0)
    assert np.isnan(got).all() and np.isfinite(ref).all()


def _lib_flag(name):
    from pypde_gb300 import _lib
    return getattr(_lib, name)
