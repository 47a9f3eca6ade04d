"""Newton-Krylov steady states (navier/rbc2d_base.py:260-341) on the GPU.

* The reference's residual semantics (``method="reference"``, the default): its
  ``steady_fun`` on a fixed sequence of points, the pressure carried from one
  evaluation to the next, against the reference's own evaluations
  (``tests/golden/golden_steady.npz``) to 1e-10; and SciPy's Newton-Krylov on it
  for 1 and 5 iterations against the reference's iterates.  A 1e-14 relative
  change of the start moves the reference's own iterate by ~1e-8 after 1 iteration
  and ~6e-8 after 5 (its residual depends on the evaluation history), so the
  iterates are compared to 1e-6.
* The augmented variant (pressure as an unknown, GPU GMRES): the converged state
  is a fixed point of the step to the requested tolerance, and of the oracle's
  step (the CPU restatement of the reference) to 1e-7.
"""
import os
import sys

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    return torch


def _start(torch, G):
    from make_golden_steady import CFG
    from pypde_gb300.navier.rbc2d import NavierStokes
    cfg = {k: v for k, v in CFG.items() if k != "beta"}
    ns = NavierStokes(beta=CFG["beta"], **cfg)
    for k in ("T", "U", "V", "pres"):
        getattr(ns, k).vhat = torch.as_tensor(G["start_" + k], device="cuda")
    return ns


def test_reference_residual_sequence_carries_the_pressure(torch):
    from make_golden_steady import DT, perturbations
    G = np.load(os.path.join(HERE, "golden", "golden_steady.npz"))
    ns = _start(torch, G)
    X0 = ns.vectorify()
    d1, d2 = (torch.as_tensor(d, device="cuda") for d in perturbations(X0.numel()))
    for k, X in enumerate((X0, X0 + d1, X0 - d2, X0)):
        F = ns.steady_fun(X.clone(), ns, None)
        assert rel_err((X + DT * F).cpu().numpy(), G["seq%d_Y" % k]) < 1e-10, k
        assert rel_err(ns.pres.vhat.cpu().numpy(), G["seq%d_pres" % k]) < 1e-10, k


@pytest.mark.parametrize("iters", [1, 5])
def test_reference_newton_krylov_iterates(torch, iters):
    G = np.load(os.path.join(HERE, "golden", "golden_steady.npz"))
    ns = _start(torch, G)
    sol = ns.solve_steady_state(X0=ns.vectorify(), tol=1e-8, maxiter=iters, disp=False)
    assert rel_err(np.asarray(sol.x), G["nk%d_x" % iters]) < 1e-6
    assert rel_err(ns.pres.vhat.cpu().numpy(), G["nk%d_pres" % iters]) < 1e-6


def test_newton_krylov_fixed_point(torch):
    from oracle import rbc2d as orb
    from pypde_gb300.navier.rbc2d import NavierStokes
    cfg = dict(case="linear", shape=(17, 17), ra=5e3, pr=1.0, dt=0.05, dealias=True, tsave=None)
    ns = NavierStokes(integrator="eu", **cfg)
    ns.set_temperature_noise(1, 1e-1)
    for _ in range(100):
        ns.update()
    res = ns.solve_steady_state(tol=1e-8, maxiter=40, disp=False, method="augmented")
    assert res.success, res.message
    # fixed point of the oracle's step with the carried pressure
    ref = orb.NavierStokes(**cfg)
    T, U, V = (x.cpu().numpy() for x in ns.reshape(res.x))
    ref.That, ref.Uhat, ref.Vhat, ref.pres = T.copy(), U.copy(), V.copy(), ns.pres.vhat.cpu().numpy().copy()
    ref.update()
    r = max(np.abs(ref.That - T).max(), np.abs(ref.Uhat - U).max(), np.abs(ref.Vhat - V).max()) / cfg["dt"]
    assert r < 1e-7, r
