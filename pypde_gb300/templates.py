"""Helmholtz / Poisson solver-plan templates (pypde/templates/{hholtz,poisson}.py)."""
import numpy as np

from .field import Field
from .host import eigdecomp
from .solver import PlanLHS, PlanRHS, SolverPlan


def _axis_mats(base):
    S = base.S
    B = base.family.B(2, 2)
    I = base.family.I(2)
    return S, B, I


def solverplan_hholtz1d(bases, lam):
    """(1 - lam D2) u = rhs + uold, premultiplied by B (hholtz.py:4-39)."""
    field = Field(bases)
    assert field.ndim == 1
    Sx, Bx, Ix = _axis_mats(field.xs[0])
    Ax = Bx @ Sx - lam * Ix @ Sx
    solver = SolverPlan()
    solver.add_rhs(PlanRHS(Bx, ndim=1, axis=0))
    solver.add_old(PlanRHS(Bx @ Sx, ndim=1, axis=0))
    solver.add_lhs(PlanLHS(Ax, ndim=1, axis=0, method="fdma"))
    return solver


def solverplan_hholtz2d_adi(bases, lam, scale=(1, 1)):
    """ADI-factored 2-D Helmholtz plan (hholtz.py:42-93)."""
    field = Field(bases)
    assert field.ndim == 2
    solver = SolverPlan()
    mats = []
    for axis in range(2):
        S, B, I = _axis_mats(field.xs[axis])
        A = B @ S - lam * (1.0 / scale[axis] ** 2.0) * I @ S
        mats.append((S, B, A))
    for axis in range(2):
        S, B, A = mats[axis]
        solver.add_rhs(PlanRHS(B, ndim=2, axis=axis))
        solver.add_old(PlanRHS(B @ S, ndim=2, axis=axis))
        solver.add_lhs(PlanLHS(A, ndim=2, axis=axis, method="fdma"))
    return solver


def solverplan_hholtz2d_fd(bases, lam, scale=(1, 1)):
    """(I - lam Laplacian) u = rhs + u_old solved exactly by fast diagonalisation in y.

    pypde has no template for this; it composes the reference's own pieces: the
    eigendecomposition of solverplan_poisson2d (poisson.py:43-110) and its Plan_Poisson
    (plans.py:254-341) with A = -lam/scale_x^2 I_x S_x, C = B_x S_x and alpha_i = 1 - lam w_i.
    rhs: B_x along x, H_y = Q_y^-1 C_y^-1 B_y along y; old: C_x along x, Q_y^-1 along y;
    lhs: the per-eigenvalue four-diagonal sweep along x (alpha_i >= 1, no singular mode), then
    Q_y along y.  Unlike solverplan_hholtz2d_adi it does not split the operator, so its result
    differs from the ADI plan's by the splitting error (lam^2 D_x^2 D_y^2 u)."""
    field = Field(bases)
    assert field.ndim == 2
    fd = poisson2d_matrices(_axis_mats(field.xs[0]), _axis_mats(field.xs[1]), False, scale)
    solver = SolverPlan()
    solver.add_rhs(PlanRHS(fd["Bx"], ndim=2, axis=0))
    solver.add_rhs(PlanRHS(fd["Hy"], ndim=2, axis=1))
    solver.add_old(PlanRHS(fd["Cx"], ndim=2, axis=0))
    solver.add_old(PlanRHS(np.linalg.inv(fd["Qy"]), ndim=2, axis=1))
    solver.add_lhs(PlanLHS(-lam * fd["Ax"], alpha=1.0 - lam * np.real(fd["wy"]), C=fd["Cx"], ndim=2, axis=0,
                           method="poisson", singular=False))
    solver.add_lhs(PlanLHS(fd["Qy"], ndim=2, axis=1, method="multiply"))
    solver._fd = fd
    return solver


def solverplan_poisson1d(bases, singular=False):
    """D2 u = rhs premultiplied by B (poisson.py:4-40)."""
    field = Field(bases)
    assert field.ndim == 1
    Sx, Bx, Ix = _axis_mats(field.xs[0])
    Ax = Ix @ Sx
    if singular:
        assert Ax[0, 0] == 0, "Matrix does not look singular"
        Ax[0, 0] += 1e-20
    solver = SolverPlan()
    solver.add_rhs(PlanRHS(Bx, ndim=1, axis=0))
    solver.add_lhs(PlanLHS(Ax, ndim=1, axis=0, method="twodma"))
    return solver


def solverplan_poisson2d(bases, singular=False, scale=(1, 1)):
    """Fast-diagonalisation 2-D Poisson plan (poisson.py:43-110)."""
    field = Field(bases)
    assert field.ndim == 2
    fd = poisson2d_matrices(_axis_mats(field.xs[0]), _axis_mats(field.xs[1]), singular, scale)
    Ax, Cx, wy, Qy, Hy, Bx = (fd[k] for k in ("Ax", "Cx", "wy", "Qy", "Hy", "Bx"))
    solver = SolverPlan()
    solver.add_rhs(PlanRHS(Bx, ndim=2, axis=0))
    solver.add_rhs(PlanRHS(Hy, ndim=2, axis=1))
    solver.add_lhs(PlanLHS(Ax, alpha=wy, C=Cx, ndim=2, axis=0, method="poisson", singular=True))
    solver.add_lhs(PlanLHS(Qy, ndim=2, axis=1, method="multiply"))
    solver._fd = fd
    return solver


def poisson2d_matrices(mx, my, singular=False, scale=(1, 1)):
    """Host matrices of the fast-diagonalisation plan (poisson.py:43-110) from the
    (S, B, I) triples of the two axes: Ax, Cx, the sorted eigenpairs wy / Qy of
    Cy^-1 Ay and the right-hand-side operator Hy = Qy^-1 Cy^-1 By."""
    Sx, Bx, Ix = mx
    Sy, By, Iy = my
    Ax = Ix @ Sx * (1.0 / scale[0] ** 2.0)
    Cx = Bx @ Sx
    Ay = Iy @ Sy * (1.0 / scale[1] ** 2.0)
    Cy = By @ Sy
    CyI = np.linalg.inv(Cy)
    wy, Qy, QyI = eigdecomp(CyI @ Ay)
    if singular:
        wy[0] += 1e-20
    Hy = QyI @ CyI @ By
    return dict(Ax=Ax, Cx=Cx, wy=wy, Qy=Qy, Hy=Hy, Bx=Bx)
