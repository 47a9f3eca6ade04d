"""Newton-Krylov steady states (navier/rbc2d_base.py:260-341) on the GPU.

The converged state must be a fixed point of the step to the requested
tolerance on the GPU, and a fixed point of the oracle's step (the CPU
restatement of the reference) to 1e-7: max |(Phi_oracle(X*) - X*) / dt|.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    return torch


def test_newton_krylov_fixed_point(torch):
    from oracle import rbc2d as orb
    from pypde_gb300.navier.rbc2d import NavierStokes
    cfg = dict(case="linear", shape=(17, 17), ra=5e3, pr=1.0, dt=0.05, dealias=True, tsave=None)
    ns = NavierStokes(integrator="eu", **cfg)
    ns.set_temperature_noise(1, 1e-1)
    for _ in range(100):
        ns.update()
    res = ns.solve_steady_state(tol=1e-8, maxiter=40, disp=False)
    assert res.success, res.message
    # fixed point of the oracle's step with the carried pressure
    ref = orb.NavierStokes(**cfg)
    T, U, V = (x.cpu().numpy() for x in ns.reshape(res.x))
    ref.That, ref.Uhat, ref.Vhat, ref.pres = T.copy(), U.copy(), V.copy(), ns.pres.vhat.cpu().numpy().copy()
    ref.update()
    r = max(np.abs(ref.That - T).max(), np.abs(ref.Uhat - U).max(), np.abs(ref.Vhat - V).max()) / cfg["dt"]
    assert r < 1e-7, r
