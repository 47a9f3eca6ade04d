"""CPU: the oracle's exact (unsplit) fast-diagonalisation Helmholtz plan and its type-2 sweep.

* HholtzFD against a dense Kronecker solve of the same premultiplied operator at small N,
  the way the reference's own test_poisson2d_kronecker.py:32-53 pins its Poisson plan.
* The band-wise type-2 sweep (diagonals of A + lam_i C formed from those of A and C) is
  bit-identical to the sweep over the dense per-eigenvalue matrices A + C*lam_i that
  solve_fdma_type2 (fdma.f90:146-185) builds.
"""
import numpy as np
import pytest

from oracle import linalg
from oracle import solver as osv
from oracle import spectral as sp


@pytest.mark.parametrize("N,M", [(33, 33), (25, 17)])
def test_exact_helmholtz_vs_kronecker(N, M):
    lam = 0.01
    f = np.random.default_rng(5).uniform(-1, 1, (N, M))
    pl = osv.HholtzFD(("CD", "CD"), (N, M), lam)
    x = pl.solve_lhs(pl.solve_rhs(f))
    Sx, Bx, Ix = sp.stencil("CD", N), sp.B2(N), sp.I2(N)
    Sy, By, Iy = sp.stencil("CD", M), sp.B2(M), sp.I2(M)
    Cx, Ax, Cy, Ay = Bx @ Sx, Ix @ Sx, By @ Sy, Iy @ Sy
    # vec(P X Q^T) = (P kron Q) vec(X) for row-major vec
    K = np.kron(Cx - lam * Ax, Cy) - lam * np.kron(Cx, Ay)
    xk = np.linalg.solve(K, (Bx @ f @ By.T).ravel()).reshape(N - 2, M - 2)
    assert np.max(np.abs(x - xk)) / np.max(np.abs(xk)) < 1e-11


def _type2_dense(A, C, lam, x, singular):
    """The type-2 sweep over the dense per-eigenvalue matrices, as the Fortran forms them."""
    x = np.array(x, dtype=np.float64)
    for i, li in enumerate(lam):
        if singular and abs(li) < 1e-10:
            l, d, u1, u2 = linalg._band4(A[1:, 1:] + C[1:, 1:] * li)
            linalg.fdma_lu(l, d, u1, u2)
            xi = x[1:, i].copy()
            linalg.fdma_solve(l, d, u1, u2, xi)
            x[1:, i] = xi
            x[0, i] = 0.0
        else:
            l, d, u1, u2 = linalg._band4(A + C * li)
            linalg.fdma_lu(l, d, u1, u2)
            xi = x[:, i].copy()
            linalg.fdma_solve(l, d, u1, u2, xi)
            x[:, i] = xi
    return x


@pytest.mark.parametrize("singular", [False, True])
def test_type2_bandwise_equals_dense(singular):
    rng = np.random.default_rng(9)
    n, m = 21, 6
    A = np.diag(rng.uniform(1, 2, n)) + np.diag(rng.uniform(-1, 1, n - 2), 2)
    C = sum(np.diag(rng.uniform(-1, 1, n - abs(k)), k) for k in (-2, 0, 2, 4))
    lam = rng.uniform(-3, 3, m)
    lam[0] = 0.0
    x = rng.uniform(-1, 1, (n, m))
    got = linalg.fdma_type2(A, C, lam, x, singular)
    ref = _type2_dense(A, C, lam, x, singular)
    assert np.array_equal(got, ref)
