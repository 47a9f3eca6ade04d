"""Pin the CPU oracle against golden vectors recorded from the reference itself.

The fixtures come from ``tests/golden/make_golden.py`` (the unmodified pypde
reference with its Fortran kernels restated as shims).  Tolerance: 1e-12
relative for single transforms / solves, 1e-9 for multi-step RBC states
(summation-order differences compound over steps).
"""
import numpy as np
import pytest

from conftest import rel_err
from oracle import field as fo
from oracle import linalg as ol
from oracle import rbc2d as orb
from oracle import solver as osv
from oracle import spectral as sp

TOL = 1e-12


@pytest.mark.parametrize("N", [33, 40, 65])
def test_chebyshev_1d(golden, N):
    f, c = golden[f"ch{N}_f"], golden[f"ch{N}_c"]
    assert rel_err(sp.cheb_forward(f, 0), golden[f"ch{N}_fwd"]) < TOL
    assert rel_err(sp.cheb_backward(c, 0), golden[f"ch{N}_bwd"]) < TOL
    assert rel_err(sp.cheb_diff(c, 1, 0), golden[f"ch{N}_d1"]) < TOL
    assert rel_err(sp.cheb_diff(c, 2, 0), golden[f"ch{N}_d2"]) < TOL


@pytest.mark.parametrize("N", [33, 40, 65])
@pytest.mark.parametrize("key", ["CD", "CN"])
def test_galerkin_1d(golden, N, key):
    f, c, v = golden[f"ch{N}_f"], golden[f"ch{N}_c"], golden[f"{key}{N}_v"]
    assert rel_err(sp.forward(key, f, 0), golden[f"{key}{N}_fwd"]) < TOL
    assert rel_err(sp.backward(key, v, 0), golden[f"{key}{N}_bwd"]) < TOL
    assert rel_err(sp.to_chebyshev(key, v, 0), golden[f"{key}{N}_toch"]) < TOL
    assert rel_err(sp.from_chebyshev(key, c, 0), golden[f"{key}{N}_fromch"]) < TOL
    assert rel_err(sp.derivative(key, v, 1, 0), golden[f"{key}{N}_d1"]) < TOL
    assert rel_err(sp.derivative(key, v, 2, 0), golden[f"{key}{N}_d2"]) < TOL


def test_dct_direct_matches_fft():
    rng = np.random.default_rng(3)
    for n in (5, 17, 33, 40):
        x = rng.uniform(-1, 1, (n, 3))
        assert rel_err(sp.dct1(x, 0), sp.dct1_direct(x, 0)) < 1e-13


@pytest.mark.parametrize("keys", [("CD", "CN"), ("CD", "CD"), ("CH", "CH")])
def test_field_2d(golden, keys):
    tag = "".join(keys)
    s = fo.Space2D(keys, (33, 20))
    g = lambda k: golden[f"f2_{tag}_{k}"]  # noqa: E731
    assert rel_err(s.forward(g("v")), g("fwd")) < TOL
    assert rel_err(s.backward(g("vh")), g("bwd")) < TOL
    assert rel_err(s.dealias_backward(g("vh")), g("dbwd")) < TOL
    assert rel_err(s.dealias_forward(g("vd")), g("dfwd")) < TOL
    for d in ((1, 0), (0, 1), (2, 0), (0, 2), (1, 1)):
        assert rel_err(fo.grad(s, g("vh"), d, (0.5, 0.25)), g(f"grad{d[0]}{d[1]}")) < TOL
    assert rel_err(fo.galerkin_to_cheby(s, g("vh")), g("g2c")) < TOL
    assert rel_err(fo.cheby_to_galerkin(s, g("ch")), g("c2g")) < TOL


@pytest.mark.parametrize("dealias", [True, False])
def test_convective_term(golden, dealias):
    t = f"conv{int(dealias)}"
    s = fo.Space2D(("CD", "CD"), (33, 20))
    d = fo.Space2D(("CH", "CH"), (33, 20))
    out = fo.convective_term(s, golden[t + "_vh"], golden[t + "_ux"], golden[t + "_uz"], d,
                             add_bc=golden[t + "_bc"], dealias=dealias, scale=(0.5, 0.5))
    assert rel_err(out, golden[t + "_out"]) < TOL


@pytest.mark.parametrize("keys", [("CD", "CD"), ("CN", "CD")])
def test_hholtz_adi(golden, keys):
    tag = "".join(keys)
    p = osv.HholtzADI(keys, (33, 25), 0.01, (0.5, 0.5))
    r = p.solve_rhs(golden[f"hh_{tag}_b"])
    assert rel_err(r, golden[f"hh_{tag}_rhs"]) < TOL
    r = r + p.solve_old(golden[f"hh_{tag}_old"])
    assert rel_err(r, golden[f"hh_{tag}_rhsold"]) < TOL
    assert rel_err(p.solve_lhs(r), golden[f"hh_{tag}_x"]) < 1e-11


@pytest.mark.parametrize("keys,singular", [(("CN", "CN"), True), (("CD", "CD"), False), (("CD", "CN"), False)])
def test_poisson(golden, keys, singular):
    tag = "".join(keys)
    p = osv.Poisson2D(keys, (33, 25), singular=singular, scale=(0.5, 0.5))
    # The intermediate H_y b depends on the eigenvector signs LAPACK picks; only
    # the solution is basis-independent, so only the solution is compared.
    x = p.solve_lhs(p.solve_rhs(golden[f"po_{tag}_b"]))
    if singular:
        x[0, 0] = 0
    assert rel_err(x, golden[f"po_{tag}_x"]) < 1e-10


def test_fdma_vs_dense_solve():
    """Independent check of the FDMA sweep (test_methods.py:71-103 pattern)."""
    rng = np.random.default_rng(11)
    N, M = 20, 10
    l, d, u1, u2 = rng.random(N - 2), rng.random(N) + 4, rng.random(N - 2), rng.random(N - 4)
    A = np.diag(d) + np.diag(u1, 2) + np.diag(u2, 4) + np.diag(l, -2)
    b = rng.random((N, M))
    fac = ol.fdma_factor(A)
    assert rel_err(ol.fdma_solve_axis(*fac, b, 0), np.linalg.solve(A, b)) < 1e-13
    assert rel_err(ol.fdma_solve_axis(*fac, b.T, 1), np.linalg.solve(A, b).T) < 1e-13
    x = b.copy()
    dd, uu = rng.random(N) + 2, rng.random(N - 2)
    ol.twodma_solve(dd, uu, x)
    assert rel_err(x, np.linalg.solve(np.diag(dd) + np.diag(uu, 2), b)) < 1e-13
    a, bb, c = rng.random(N - 2), rng.random(N) + 3, rng.random(N - 2)
    T = np.diag(a, -2) + np.diag(bb) + np.diag(c, 2)
    assert rel_err(ol.tdma_offset(a, bb, c, b, 2), np.linalg.solve(T, b)) < 1e-13


CASES = [
    ("rbc_lin33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 10, 0, 1e-2),
    ("rbc_lin33nd", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=False, integrator="eu"), 10, 0, 1e-2),
    ("rbc_lin33x17", "linear", (33, 17), dict(ra=3e4, dt=0.01, dealias=True, integrator="eu", aspect=2.0), 10, 5, 1e-2),
    ("rbc_rbc33", "rbc", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 10, 1, 1e-2),
    ("rbc_zero33", "zero", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 10, 2, 1e-2),
    ("rbc_rk3_33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="rk3"), 5, 3, 1e-2),
    ("rbc_beta33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu", beta=0.5), 5, 4, 1e-2),
    ("rbc_c1", "linear", (65, 65), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 100, 0, 1e-3),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_rbc2d_steps(golden, case):
    tag, kind, shape, cfg, nsteps, seed, amp = case
    ns = orb.NavierStokes(case=kind, shape=shape, pr=1.0, tsave=None, **cfg)
    orb.seeded_temperature(ns, seed, amp)
    assert rel_err(ns.That, golden[tag + "_T0"]) < TOL
    for _ in range(nsteps):
        ns.update()
    st = f"{tag}_s{nsteps}"
    for name, arr in (("T", ns.That), ("U", ns.Uhat), ("V", ns.Vhat), ("P", ns.Phat), ("pres", ns.pres)):
        assert rel_err(arr, golden[f"{st}_{name}"]) < 1e-9, name
    nu, nuv, ke = golden[st + "_scalars"]
    assert abs(ns.eval_Nu() - nu) / abs(nu) < 1e-10
    assert abs(ns.eval_Nuvol() - nuv) / abs(nuv) < 1e-10
    assert abs(ns.eval_KE() - ke) / abs(ke) < 1e-8


def test_adjoint_step(golden):
    """One adjoint-descent step (navier/rbc2d_adj.py) against the reference's own output."""
    from oracle import rbc2d_adj as oadj
    nsa = oadj.NavierStokesAdjoint(case="linear", shape=(33, 33), ra=1e5, pr=1.0, dt=0.01, tsave=None,
                                   dealias=True, integrator="eu", beta=1.0)
    noise = 1e-2 * np.random.default_rng(7).uniform(-1, 1, (33, 33))
    nsa.That = nsa.Tsp.forward(noise)
    assert rel_err(nsa.That, golden["adj33_T0"]) < TOL
    nsa.update()
    for name, arr in (("T1", nsa.That), ("U1", nsa.Uhat), ("V1", nsa.Vhat), ("FT", nsa.FT), ("FU", nsa.FU),
                      ("FV", nsa.FV), ("TA", nsa.TA), ("UA", nsa.UA), ("VA", nsa.VA)):
        assert rel_err(arr, golden["adj33_" + name]) < 1e-9, name
