"""Solver plans restated in NumPy (oracle, test infrastructure).

Reference: pypde/templates/hholtz.py, pypde/templates/poisson.py,
pypde/solver/plans.py, pypde/solver/solverplan.py, pypde/solver/matrix.py,
pypde/solver/utils.py.
"""
import numpy as np
import scipy.sparse

from . import spectral as sp
from . import linalg


def apply_along(A, b, axis):
    """PlanRHS.solve -> MatrixBase.dot with a CSR matrix (plans.py:54-74, matrix.py:41-56)."""
    A = scipy.sparse.csr_matrix(A)
    if axis == 0:
        return np.asarray(A @ b)
    return np.swapaxes(np.asarray(A @ np.swapaxes(b, axis, 0)), axis, 0)


def eigdecomp(A):
    """eigdecomp (solver/utils.py:13-29): eigenpairs sorted by descending eigenvalue."""
    w, Q = np.linalg.eig(A)
    order = np.argsort(w)[::-1]
    w = w[order]
    Q = Q[:, order]
    return w, Q, np.linalg.inv(Q)


class HholtzADI:
    """solverplan_hholtz2d_adi (hholtz.py:42-93) for bases ``keys`` on ``shape``.

    (I - lam D^2) u = rhs + u_old, premultiplied by the pseudo-inverse B and
    ADI-factored: rhs plans B (x), B (y); old plans B S (x), B S (y);
    lhs FDMA(A_x) along x then FDMA(A_y) along y.
    """

    def __init__(self, keys, shape, lam, scale=(1.0, 1.0)):
        self.B, self.BS, self.fac = [], [], []
        for axis in range(2):
            N = shape[axis]
            S = sp.stencil(keys[axis], N)
            B = sp.B2(N)
            I = sp.I2(N)
            A = B @ S - lam * (1.0 / scale[axis] ** 2.0) * I @ S
            self.B.append(B)
            self.BS.append(B @ S)
            self.fac.append(linalg.fdma_factor(A))

    def solve_rhs(self, b):
        for axis in range(2):
            b = apply_along(self.B[axis], b, axis)
        return b

    def solve_old(self, b):
        for axis in range(2):
            b = apply_along(self.BS[axis], b, axis)
        return b

    def solve_lhs(self, b):
        for axis in range(2):
            b = linalg.fdma_solve_axis(*self.fac[axis], b, axis)
        return b


class Poisson2D:
    """solverplan_poisson2d (poisson.py:43-110): fast diagonalisation in y.

    rhs plans: B_x along x, H_y = Q_y^-1 C_y^-1 B_y along y;
    lhs: per-eigenvalue FDMA type-2 along x (always singular=True, poisson.py:106),
    then Q_y along y.
    """

    def __init__(self, keys, shape, singular=False, scale=(1.0, 1.0)):
        Nx, Ny = shape
        Sx, Sy = sp.stencil(keys[0], Nx), sp.stencil(keys[1], Ny)
        Bx, By = sp.B2(Nx), sp.B2(Ny)
        Ix, Iy = sp.I2(Nx), sp.I2(Ny)
        self.Ax = Ix @ Sx * (1.0 / scale[0] ** 2.0)
        self.Cx = Bx @ Sx
        Ay = Iy @ Sy * (1.0 / scale[1] ** 2.0)
        Cy = By @ Sy
        CyI = np.linalg.inv(Cy)
        wy, Qy, QyI = eigdecomp(CyI @ Ay)
        if singular:
            wy[0] += 1e-20
        self.wy = np.real(wy)
        self.Hy = np.real(QyI @ CyI @ By)
        self.Qy = np.real(Qy)
        self.Bx = Bx

    def solve_rhs(self, b):
        b = apply_along(self.Bx, b, 0)
        return apply_along(self.Hy, b, 1)

    def solve_lhs(self, b):
        x = linalg.fdma_type2(self.Ax, self.Cx, self.wy, b, singular=True)
        return apply_along(self.Qy, x, 1)


class HholtzFD:
    """(I - lam Laplacian) u = rhs + u_old by fast diagonalisation in y, exactly (no ADI splitting).

    The reference's Plan_Poisson (plans.py:254-341, solve_fdma_type2 of fdma.f90:146-185) with
    A = -lam/scale_x^2 I_x S_x, C = B_x S_x and alpha_i = 1 - lam w_i, where w, Q_y are the
    eigenpairs of C_y^-1 I_y S_y / scale_y^2 that solverplan_poisson2d builds (poisson.py:43-110):
    rhs plans B_x along x, H_y = Q_y^-1 C_y^-1 B_y along y; old plans C_x along x, Q_y^-1 along y;
    lhs the per-eigenvalue type-2 sweep along x (no singular mode: alpha_i >= 1), then Q_y along y.
    """

    def __init__(self, keys, shape, lam, scale=(1.0, 1.0)):
        po = Poisson2D(keys, shape, singular=False, scale=scale)
        self.A = -lam * po.Ax
        self.C = po.Cx
        self.alpha = 1.0 - lam * po.wy
        self.Bx, self.Hy, self.Qy = po.Bx, po.Hy, po.Qy
        self.QyI = np.linalg.inv(po.Qy)

    def solve_rhs(self, b):
        b = apply_along(self.Bx, b, 0)
        return apply_along(self.Hy, b, 1)

    def solve_old(self, b):
        b = apply_along(self.C, b, 0)
        return apply_along(self.QyI, b, 1)

    def solve_lhs(self, b):
        x = linalg.fdma_type2(self.A, self.C, self.alpha, b, singular=False)
        return apply_along(self.Qy, x, 1)
