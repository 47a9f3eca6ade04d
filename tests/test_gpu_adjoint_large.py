"""GPU: adjoint-descent step (navier/rbc2d_adj.py) and large-grid parity (513 x 257, 257^2)."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    return torch


def host(t):
    return t.detach().cpu().numpy()


def test_adjoint_step_golden(torch, golden):
    from pypde_gb300.navier.rbc2d_adj import NavierStokesAdjoint
    nsa = NavierStokesAdjoint(case="linear", shape=(33, 33), ra=1e5, pr=1.0, dt=0.01, tsave=None, dealias=True,
                              integrator="eu", beta=1.0)
    nsa.T.v = 1e-2 * np.random.default_rng(7).uniform(-1, 1, (33, 33))
    nsa.T.forward()
    assert rel_err(host(nsa.T.vhat), golden["adj33_T0"]) < 1e-10
    nsa.update()
    got = {"T1": nsa.T.vhat, "U1": nsa.U.vhat, "V1": nsa.V.vhat, "FT": nsa.NS.T.vhat, "FU": nsa.NS.U.vhat,
           "FV": nsa.NS.V.vhat, "TA": nsa.TA.vhat, "UA": nsa.UA.vhat, "VA": nsa.VA.vhat}
    for name, t in got.items():
        assert rel_err(host(t), golden["adj33_" + name]) < 1e-9, name


def test_adjoint_steps_vs_oracle_rbc(torch):
    from oracle import rbc2d_adj as oadj
    from pypde_gb300.navier.rbc2d_adj import NavierStokesAdjoint
    kw = dict(case="rbc", shape=(33, 49), ra=5e4, pr=1.0, dt=0.02, tsave=None, dealias=True, integrator="eu")
    ref = oadj.NavierStokesAdjoint(**kw)
    nsa = NavierStokesAdjoint(**kw)
    noise = 1e-2 * np.random.default_rng(12).uniform(-1, 1, (33, 49))
    ref.That = ref.Tsp.forward(noise)
    nsa.T.v = noise
    nsa.T.forward()
    for _ in range(3):
        ref.update()
        nsa.update()
    for name, a, b in (("T", nsa.T.vhat, ref.That), ("U", nsa.U.vhat, ref.Uhat), ("V", nsa.V.vhat, ref.Vhat),
                       ("TA", nsa.TA.vhat, ref.TA), ("UA", nsa.UA.vhat, ref.UA)):
        assert rel_err(host(a), b) < 1e-8, name


def test_large_plain_513x257_fused_vs_oracle(torch):
    """The large configuration (513 x 257, aspect 2, Ra 1e8, dt 1e-3, 3/2 dealiasing): 2 fused steps."""
    from oracle import rbc2d as orb
    from pypde_gb300.navier.rbc2d import NavierStokes
    kw = dict(case="linear", shape=(513, 257), ra=1e8, pr=1.0, dt=1e-3, aspect=2.0, dealias=True, integrator="eu",
              tsave=None)
    ref = orb.NavierStokes(**kw)
    orb.seeded_temperature(ref, 2, 1e-3)
    ns = NavierStokes(**kw)
    ns.set_temperature_noise(2, 1e-3)
    f = ns.fused()
    for _ in range(2):
        ref.update()
        f.step_eager()
    st = ns.state()
    for name, arr in (("T", ref.That), ("U", ref.Uhat), ("V", ref.Vhat), ("P", ref.Phat), ("pres", ref.pres)):
        assert rel_err(st[name], arr) < 1e-8, name


@pytest.mark.parametrize("N", [257])
def test_helmholtz_adi_257(torch, N):
    """(I - 0.01 Laplacian) u = f, Dirichlet bases, N x N, f ~ U(-1,1) (seed 1): ADI plan vs oracle, and the
    residual of the ADI-factored operator applied to the solution."""
    import pypde_gb300 as pg
    from oracle import solver as osv
    rng = np.random.default_rng(1)
    f = rng.uniform(-1, 1, (N, N))
    ref = osv.HholtzADI(("CD", "CD"), (N, N), 0.01)
    x_ref = ref.solve_lhs(ref.solve_rhs(f))
    fld = pg.Field([pg.Base(N, "CD"), pg.Base(N, "CD")])
    sol = pg.solverplan_hholtz2d_adi(fld.xs, lam=0.01)
    x = host(sol.solve_lhs(sol.solve_rhs(f)))
    assert rel_err(x, x_ref) < 1e-10
    # residual: A_y (A_x x) == B_y B_x f along the respective axes (the ADI-factored system)
    from oracle import spectral as sp
    S, B, I = sp.stencil("CD", N), sp.B2(N), sp.I2(N)
    A = B @ S - 0.01 * I @ S
    lhs = A @ x @ A.T
    rhs = B @ f @ B.T
    assert np.max(np.abs(lhs - rhs)) / np.max(np.abs(rhs)) < 1e-12
