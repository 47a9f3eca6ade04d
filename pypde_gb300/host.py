"""Setup-time operator matrices (host, FP64), built once per plan.

These are the small matrices pypde builds with NumPy before any time step:
Gauss-Lobatto grid (dmsuite.py:209-214), Shen stencils (chebyshev.py:382-392,
426-436, 555-559, 586-590), the banded pseudo-inverse of the Chebyshev D^2
(dmsuite.py:327-368), the four-diagonal LU sweep (plans.py:226-234) and the
sorted eigendecomposition of the fast-diagonalisation Poisson plan
(solver/utils.py:13-29).  Nothing here runs inside a time step.
"""
import numpy as np


def gauss_lobatto(n):
    """n+1 Chebyshev-Gauss-Lobatto points x_j = -cos(pi j / n), ascending."""
    if n <= 1:
        return 0
    j = np.arange(n, -1, -1, dtype=np.float64)
    return np.sin(np.pi * (n - 2.0 * j) / (2.0 * n))


def dealias_size(N, factor=1.5):
    return int(N * factor)


def stencil_sub(key, N):
    """Sub-diagonal S[i+2, i] (i < N-2) of a Shen stencil with S[i, i] = 1."""
    i = np.arange(N - 2, dtype=np.float64)
    if key == "CD":
        return -np.ones(N - 2)
    if key == "CN":
        return -((i / (i + 2.0)) ** 2)
    raise ValueError(key)


def stencil_matrix(key, N):
    """Stencil S (N x M) mapping Galerkin to Chebyshev coefficients."""
    if key in ("CD", "CN"):
        S = np.zeros((N, N - 2))
        k = np.arange(N - 2)
        S[k, k] = 1.0
        S[k + 2, k] = stencil_sub(key, N)
        return S
    S = np.zeros((N, 2))
    if key == "DC":
        S[:2, :] = [[0.5, 0.5], [-0.5, 0.5]]
    elif key == "NC":
        S[:2, :] = [[0.5, 0.5], [-1.0 / 8.0, 1.0 / 8.0]]
    else:
        raise ValueError(key)
    return S


def pseudoinverse_d2(N):
    """Banded (offsets -2, 0, +2) pseudo-inverse of the Chebyshev second-derivative matrix."""
    P = np.zeros((N, N))
    i = np.arange(2, N - 2)
    P[i, i] = -1.0 / (2.0 * (i * i - 1.0))
    i = np.arange(2, N - 4)
    P[i, i + 2] = 1.0 / (4.0 * i * (i + 1.0))
    i = np.arange(2, N)
    P[i, i - 2] = 1.0 / (4.0 * i * (i - 1.0))
    P[2, 0] *= 2.0
    P[np.abs(P) < 1e-12] = 0.0
    return P


def fdma_lu(A):
    """Diagonals (-2, 0, +2, +4) of A and their in-place LU sweep, as Plan_fdma does."""
    l = np.diag(A, -2).astype(np.float64).copy()
    d = np.diag(A, 0).astype(np.float64).copy()
    u1 = np.diag(A, 2).astype(np.float64).copy()
    u2 = np.diag(A, 4).astype(np.float64).copy()
    n = d.shape[0]
    for i in range(2, n):
        l[i - 2] = l[i - 2] / d[i - 2]
        d[i] = d[i] - l[i - 2] * u1[i - 2]
        if i < n - 2:
            u1[i] = u1[i] - l[i - 2] * u2[i - 2]
    return l, d, u1, u2


def eigdecomp(A):
    """Eigenpairs sorted by descending (real) eigenvalue, plus the inverse eigenvector matrix."""
    w, Q = np.linalg.eig(A)
    if np.iscomplexobj(w) and np.all(w.imag == 0.0):
        w, Q = w.real, Q.real
    order = np.argsort(w)[::-1]
    w, Q = w[order], Q[:, order]
    return w, Q, np.linalg.inv(Q)
