"""Transposed kernels and the discrete adjoint of the time step.

Each device operator A is checked by materialising it (A applied to the
identity, through the forward kernel that the parity tests pin to the oracle)
and comparing the autograd backward, which runs the hand-written transposed
kernel, with A^T y: 1e-12 relative.  The step's gradient is checked against
central finite differences, h = 1e-6: 1e-6 relative (the path's stated target),
once with the GPU forward map and once with the oracle's forward map on the CPU.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_T = 1e-12


@pytest.fixture(scope="module")
def pg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    import pypde_gb300
    return pypde_gb300


def _check_transpose(fwd, n_in, n_out, lines=7, seed=0):
    """backward of fwd along axis 0 == A^T, A = fwd(I); also along axis 1 through views."""
    import torch
    A = fwd(torch.eye(n_in, dtype=torch.float64, device="cuda"))
    assert A.shape == (n_out, n_in)
    rng = np.random.default_rng(seed)
    x = torch.as_tensor(rng.standard_normal((n_in, lines)), device="cuda").requires_grad_(True)
    y = torch.as_tensor(rng.standard_normal((n_out, lines)), device="cuda")
    (g,) = torch.autograd.grad(fwd(x), x, y)
    ref = A.T @ y
    err = float((g - ref).abs().max() / ref.abs().max())
    assert err < TOL_T, err
    # axis 1: the same operator on a transposed view
    xt = x.detach().T.contiguous().requires_grad_(True)
    (gt,) = torch.autograd.grad(fwd(xt.T).T, xt, y.T.contiguous())
    err = float((gt.T - ref).abs().max() / ref.abs().max())
    assert err < TOL_T, err


DCT_CASES = [(33, 33, 33), (65, 65, 65), (129, 129, 129), (1025, 1025, 1025), (49, 49, 49), (97, 65, 65),
             (97, 97, 65), (28, 28, 28), (10, 7, 10), (40, 40, 40), (50, 33, 50), (17, 12, 17), (3, 3, 3)]


@pytest.mark.parametrize("N,n_in,n_out", DCT_CASES, ids=[f"{c[0]}-{c[1]}-{c[2]}" for c in DCT_CASES])
@pytest.mark.parametrize("which", ["fwd", "bwd"])
def test_dct_transposes(pg, N, n_in, n_out, which):
    """Even-folded FFT (N-1 even, 2^a 3^b), paired-line FFT (N-1 odd) and dense-matrix lengths,
    with zero padding of the input and truncation of the output."""
    from pypde_gb300 import _lib
    CH = pg.Base(N, "CH")
    mode = _lib.DCT_FWD if which == "fwd" else _lib.DCT_BWD
    _check_transpose(lambda x: CH._dct(x, mode, n_out), n_in, n_out)


@pytest.mark.parametrize("N", [33, 65, 64, 257])
@pytest.mark.parametrize("deriv", [1, 2])
def test_derivative_transpose(pg, N, deriv):
    CH = pg.Base(N, "CH")
    _check_transpose(lambda x: CH.derivative(x, deriv), N, N)


@pytest.mark.parametrize("N", [33, 64, 129])
@pytest.mark.parametrize("key", ["CD", "CN"])
def test_stencil_transposes(pg, N, key):
    B = pg.Base(N, key)
    _check_transpose(B.to_chebyshev, N - 2, N)
    _check_transpose(B.from_chebyshev, N, N - 2)
    _check_transpose(lambda x: B.derivative(x, 1), N - 2, N)


def test_matrix_and_bc_transposes(pg):
    from pypde_gb300.bases import MatrixApply
    CH = pg.Base(33, "CH")
    rng = np.random.default_rng(5)
    for A in (CH.B(2, 2), CH.B(2, 2) @ pg.Base(33, "CD").S, rng.standard_normal((9, 33))):
        M = MatrixApply(A)
        _check_transpose(lambda x: M.apply(x, 0), A.shape[1], A.shape[0])
    DC = pg.Base(33, "CD").bc
    _check_transpose(DC.to_chebyshev, 2, 33)
    _check_transpose(DC.from_chebyshev, 33, 2)


def test_banded_solve_transposes(pg):
    from pypde_gb300.solver import Plan_fdma
    from pypde_gb300.templates import solverplan_hholtz2d_adi, solverplan_poisson1d
    for key, N in (("CD", 33), ("CN", 65), ("CD", 129)):
        s = solverplan_hholtz2d_adi([pg.Base(N, key), pg.Base(N, "CD")], lam=0.013, scale=(1.0, 0.5))
        plan = s.plan_for_lhs[0]
        assert isinstance(plan, Plan_fdma)
        _check_transpose(lambda x: plan.solve(x), N - 2, N - 2)
    import torch
    s = solverplan_poisson1d([pg.Base(33, "CD")])
    two = s.plan_for_lhs[0]
    _check_transpose(lambda x: torch.stack([two.solve(x[:, j].clone()) for j in range(x.shape[1])], 1), 31, 31)


@pytest.mark.parametrize("singular", [False, True])
@pytest.mark.parametrize("keys", [("CD", "CD"), ("CN", "CN")])
def test_poisson_transposes(pg, singular, keys):
    import torch
    from pypde_gb300.templates import solverplan_poisson2d
    N, M = 33, 17
    s = solverplan_poisson2d([pg.Base(N, keys[0]), pg.Base(M, keys[1])], singular=singular, scale=(1.0, 0.5))
    plan = s.plan_for_lhs[0]
    n, m = N - 2, M - 2
    rng = np.random.default_rng(9)
    x = torch.as_tensor(rng.standard_normal((n, m)), device="cuda").requires_grad_(True)
    y = torch.as_tensor(rng.standard_normal((n, m)), device="cuda")
    (g,) = torch.autograd.grad(plan.solve(x), x, y)
    # reference: for every eigenvalue column j, (A + w_j C)^-T y_j (singular rule: row/col 0 dropped)
    A, C, w = s._fd["Ax"], s._fd["Cx"], np.real(s._fd["wy"])
    yh, ref = y.cpu().numpy(), np.zeros((n, m))
    for j in range(m):
        K = A + w[j] * C
        if abs(w[j]) < 1e-10:  # the plan always applies the singular rule (poisson.py:106)
            ref[1:, j] = np.linalg.solve(K[1:, 1:].T, yh[1:, j])
        else:
            ref[:, j] = np.linalg.solve(K.T, yh[:, j])
    err = float(np.abs(g.cpu().numpy() - ref).max() / np.abs(ref).max())
    assert err < 1e-11, err


def test_double_backward_is_forward(pg):
    """The backward of the backward is the forward operator: grad of <A^T y, v> w.r.t. y is A v."""
    import torch
    from pypde_gb300 import _lib
    CH = pg.Base(65, "CH")
    rng = np.random.default_rng(2)
    x = torch.as_tensor(rng.standard_normal((65, 4)), device="cuda").requires_grad_(True)
    y = torch.as_tensor(rng.standard_normal((65, 4)), device="cuda").requires_grad_(True)
    v = torch.as_tensor(rng.standard_normal((65, 4)), device="cuda")
    (g,) = torch.autograd.grad(CH._dct(x, _lib.DCT_FWD), x, y, create_graph=True)
    (gy,) = torch.autograd.grad(g, y, v)
    ref = CH._dct(v, _lib.DCT_FWD)
    assert float((gy - ref).abs().max() / ref.abs().max()) < TOL_T


def _ns(case, shape, **kw):
    from pypde_gb300.navier.rbc2d import NavierStokes
    cfg = dict(ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu", tsave=None)
    cfg.update(kw)
    return NavierStokes(case=case, shape=shape, **cfg)


@pytest.mark.parametrize("case,shape,dealias", [("linear", (33, 33), True), ("rbc", (33, 17), True),
                                                ("linear", (24, 20), False)])
def test_step_gradient_vs_finite_differences(pg, case, shape, dealias):
    """J = ||Phi^12(X) - X|| with checkpoints every 5 steps, 3 random unit directions, h = 1e-6."""
    from pypde_gb300.navier.adjoint import ResidualObjective, fd_check, random_directions
    ns = _ns(case, shape, dealias=dealias)
    ns.set_temperature_noise(3, 1e-2)
    import torch
    rng = np.random.default_rng(4)
    du = torch.as_tensor(rng.uniform(-1, 1, tuple(ns.U.vhat.shape)), device="cuda")
    X = (ns.T.vhat.clone(), ns.U.vhat + 1e-3 * du, ns.V.vhat.clone())
    obj = ResidualObjective(ns, nsteps=12, every=5)
    dirs = random_directions([x.shape for x in X], 3, seed=11, device="cuda")
    J, rows = fd_check(obj, X, dirs, h=1e-6)
    assert J > 0
    for fd, ad, err in rows:
        assert err < 1e-6, (fd, ad, err)


def test_step_gradient_vs_oracle_finite_differences(pg):
    """Directional derivative of the oracle's J (CPU, central differences) against the GPU adjoint."""
    from oracle import rbc2d as orb
    from pypde_gb300.navier.adjoint import ResidualObjective, random_directions
    shape, nsteps = (33, 33), 6
    ns = _ns("linear", shape)
    ns.set_temperature_noise(3, 1e-2)
    X = (ns.T.vhat.clone(), ns.U.vhat.clone(), ns.V.vhat.clone())
    (d,) = random_directions([x.shape for x in X], 1, seed=12, device="cuda")
    J, g = ResidualObjective(ns, nsteps=nsteps, every=4).value_and_grad(X)
    ad = float(sum((gi * e).sum() for gi, e in zip(g, d)))
    ref = orb.NavierStokes(case="linear", shape=shape, ra=1e5, pr=1.0, dt=0.01, dealias=True, tsave=None)
    Xh = [x.cpu().numpy() for x in X]
    dh = [e.cpu().numpy() for e in d]

    def J_oracle(sign, h=1e-6):
        ref.That, ref.Uhat, ref.Vhat = [x + sign * h * e for x, e in zip(Xh, dh)]
        ref.pres = np.zeros_like(ref.pres)
        X0 = (ref.That.copy(), ref.Uhat.copy(), ref.Vhat.copy())
        for _ in range(nsteps):
            ref.update()
        return np.sqrt(sum(((a - b) ** 2).sum() for a, b in zip((ref.That, ref.Uhat, ref.Vhat), X0)))

    assert abs(J_oracle(0) - J) / J < 1e-8
    fd = (J_oracle(+1) - J_oracle(-1)) / 2e-6
    assert abs(fd - ad) / abs(ad) < 1e-6, (fd, ad)


def test_rbc2d_adj_direction_vs_discrete_gradient(pg):
    """pypde's adjoint-descent direction (navier/rbc2d_adj.py: continuous adjoint of the one-step residual
    F = (Phi(X) - X)/dt, smoothed by an inverse Laplacian, plus F itself) and the exact discrete gradient of
    J1 = |F|^2 / 2 are different quantities; measured on 33 x 33, Ra 1e4, dt 1e-2 the reference's direction
    is nearly F (cosine 0.997) and has cosine 0.92 with -grad J1 (0.53 - 0.92 over Ra 1e4 - 1e5, dt 1e-4 - 1e-2)."""
    import torch
    from pypde_gb300.navier.adjoint import step
    from pypde_gb300.navier.rbc2d_adj import NavierStokesAdjoint
    cfg = dict(shape=(33, 33), ra=1e4, pr=1.0, dt=1e-2, dealias=True, integrator="eu", tsave=None)
    A = NavierStokesAdjoint(case="linear", **cfg)
    rng = np.random.default_rng(0)
    A.T.vhat = torch.as_tensor(1e-2 * rng.uniform(-1, 1, tuple(A.T.vhat.shape)), device="cuda")
    A.U.vhat = torch.as_tensor(1e-3 * rng.uniform(-1, 1, tuple(A.U.vhat.shape)), device="cuda")
    A.V.vhat = torch.as_tensor(1e-3 * rng.uniform(-1, 1, tuple(A.V.vhat.shape)), device="cuda")
    X = [A.T.vhat.clone(), A.U.vhat.clone(), A.V.vhat.clone()]
    A.update()
    dt = cfg["dt"]
    D = [(A.T.vhat - X[0]) / dt, (A.U.vhat - X[1]) / dt, (A.V.vhat - X[2]) / dt]
    ns = _ns("linear", (33, 33), ra=1e4, dt=dt)
    Xr = [x.clone().requires_grad_(True) for x in X]
    with torch.enable_grad():
        Y = step(ns, (*Xr, torch.zeros_like(ns.pres.vhat)))
        F = [(y - x) / dt for y, x in zip(Y[:3], Xr)]
        g = torch.autograd.grad(0.5 * sum((f * f).sum() for f in F), Xr)

    def cos(a, b):
        num = sum(float((x * y).sum()) for x, y in zip(a, b))
        return num / np.sqrt(sum(float((x * x).sum()) for x in a) * sum(float((y * y).sum()) for y in b))

    assert cos(D, [f.detach() for f in F]) > 0.99
    assert cos(D, [-x for x in g]) > 0.85
