"""Banded sweeps restated from the reference's Fortran kernels (oracle, test infrastructure).

Reference: pypde/bases/linalg/fortran/tdma.f90, pypde/solver/linalg/fortran/fdma.f90,
pypde/solver/linalg/fortran/twodma.f90, pypde/solver/plans.py.  The sweeps run
along axis 0 and are vectorised over the remaining axes, exactly as the
Fortran whole-row array statements are.  0-based indices throughout.
"""
import numpy as np

from . import _ck


def tdma_offset(a, b, c, d, k):
    """solve_tdma_2d (tdma.f90:56-107): A x = d, A banded at offsets -k, 0, +k.

    a: n-k (offset -k), b: n (diagonal), c: n-k (offset +k), d: n x ... rhs.
    """
    d = np.asarray(d, dtype=np.float64)
    n = b.shape[0]
    L = _ck.lib()
    if L is not None and n > k:
        dd = _ck.c64(d.reshape(n, -1))
        m = dd.shape[1]
        g, x, w = np.empty_like(dd), np.empty_like(dd), np.zeros(n - k)
        a, b, c = _ck.c64(a), _ck.c64(b), _ck.c64(c)
        L.ok_tdma_offset(_ck.ptr(a), _ck.ptr(b), _ck.ptr(c), _ck.ptr(dd), _ck.ptr(x), _ck.ptr(g), _ck.ptr(w), n, m, k)
        return x.reshape(d.shape)
    w = np.zeros(n - k)
    for i in range(n - k):
        w[i] = c[i] / b[i] if i < k else c[i] / (b[i] - a[i - k] * w[i - k])
    g = np.empty_like(d)
    for i in range(n):
        if i < k:
            g[i] = d[i] / b[i]
        else:
            g[i] = (d[i] - a[i - k] * g[i - k]) / (b[i] - a[i - k] * w[i - k])
    x = np.empty_like(d)
    x[n - k - 1:] = g[n - k - 1:]
    for j in range(n - k - 1, -1, -1):
        x[j] = g[j] - w[j] * x[j + k]
    return x


def fdma_lu(l, d, u1, u2):
    """Plan_fdma.FDMA_LU (plans.py:226-234) == init_fdma's sweep (fdma.f90:135-141), in place."""
    n = d.shape[0]
    L = _ck.lib()
    if L is not None and d.ndim == 2 and n >= 4 and all(v.flags.c_contiguous and v.dtype == np.float64
                                                         for v in (l, d, u1, u2)):
        L.ok_fdma_lu(_ck.ptr(l), _ck.ptr(d), _ck.ptr(u1), _ck.ptr(u2), n, d.shape[1])
        return l, d, u1, u2
    for i in range(2, n):
        l[i - 2] = l[i - 2] / d[i - 2]
        d[i] = d[i] - l[i - 2] * u1[i - 2]
        if i < n - 2:
            u1[i] = u1[i] - l[i - 2] * u2[i - 2]
    return l, d, u1, u2


def fdma_factor(A):
    """Extract diagonals -2, 0, +2, +4 of A and LU-sweep them (plans.py:193-199)."""
    l = np.diag(A, -2).copy()
    d = np.diag(A, 0).copy()
    u1 = np.diag(A, 2).copy()
    u2 = np.diag(A, 4).copy()
    return fdma_lu(l, d, u1, u2)


def fdma_solve(l, d, u1, u2, x):
    """solve_fdma_1d / solve_fdma_2d along axis 0 (fdma.f90:1-38, 68-81), in place on x."""
    n = d.shape[0]
    L = _ck.lib()
    if L is not None and n >= 4:
        cs = 1 if d.ndim == 2 else 0
        xx = _ck.c64(x.reshape(n, -1))
        m = xx.shape[1]
        if not cs or d.shape[1] == m:
            co = [_ck.c64(v) for v in (l, d, u1, u2)]
            L.ok_fdma_solve(*[_ck.ptr(v) for v in co], cs, _ck.ptr(xx), n, m)
            if not np.shares_memory(xx, x):
                x[...] = xx.reshape(x.shape)
            return x
    for i in range(2, n):
        x[i] -= l[i - 2] * x[i - 2]
    x[n - 1] = x[n - 1] / d[n - 1]
    x[n - 2] = x[n - 2] / d[n - 2]
    x[n - 3] = (x[n - 3] - u1[n - 3] * x[n - 1]) / d[n - 3]
    x[n - 4] = (x[n - 4] - u1[n - 4] * x[n - 2]) / d[n - 4]
    for i in range(n - 5, -1, -1):
        x[i] = (x[i] - u1[i] * x[i + 2] - u2[i] * x[i + 4]) / d[i]
    return x


def fdma_solve_axis(l, d, u1, u2, x, axis):
    """solve_fdma_2d with ``axis`` 0 or 1 (fdma.f90:40-98); returns the solved array."""
    xs = np.array(np.moveaxis(x, axis, 0), dtype=np.float64)
    fdma_solve(l, d, u1, u2, xs)
    return np.moveaxis(xs, 0, axis)


def twodma_solve(d, u, x):
    """solve_twodma_1d / _2d along axis 0 (twodma.f90:2-62), in place on x."""
    n = d.shape[0]
    L = _ck.lib()
    if L is not None and n >= 2:
        xx = _ck.c64(x.reshape(n, -1))
        d, u = _ck.c64(d), _ck.c64(u)
        L.ok_twodma_solve(_ck.ptr(d), _ck.ptr(u), _ck.ptr(xx), n, xx.shape[1])
        if not np.shares_memory(xx, x):
            x[...] = xx.reshape(x.shape)
        return x
    x[n - 1] = x[n - 1] / d[n - 1]
    x[n - 2] = x[n - 2] / d[n - 2]
    for i in range(n - 3, -1, -1):
        x[i] = (x[i] - u[i] * x[i + 2]) / d[i]
    return x


def _band4(A):
    """Diagonals d, l(-2), u1(+2), u2(+4) of a square (stack of) matrices, zero-padded
    to full length like init_fdma's zero initialisation (fdma.f90:124-133)."""
    def diag(k):  # rows first: (n - |k|, ...) C-contiguous
        return np.ascontiguousarray(np.moveaxis(np.diagonal(A, k, -2, -1), -1, 0))
    return diag(-2), diag(0), diag(2), diag(4)


def fdma_type2(A, C, lam, x, singular):
    """solve_fdma_type2, axis 0 (fdma.f90:146-185): (A + lam_i C) x_i = b_i per column i.

    For each column the 4 diagonals of A + lam_i*C are LU-swept (init_fdma,
    fdma.f90:102-143) and solved (solve_fdma_1d).  When ``singular`` and
    |lam_i| < 1e-10 the system is solved on rows/cols 1: and x_0 = 0.
    Vectorised over columns; returns a new array.
    """
    x = np.array(x, dtype=np.float64)
    lam = np.real(np.asarray(lam))
    n, m = x.shape
    sing = np.zeros(m, dtype=bool)
    if singular:
        sing = np.abs(lam) < 1e-10
    reg = ~sing
    # the four diagonals of A + C*lam_i, element for element the Fortran's A(i,j) + C(i,j)*lam(i),
    # formed from the diagonals of A and C (no dense matrix per eigenvalue)
    bA, bC = _band4(A), _band4(C)

    def band(lams, first):
        return [np.ascontiguousarray(a[first:, None] + c[first:, None] * lams[None, :]) for a, c in zip(bA, bC)]

    if reg.any():
        l, d, u1, u2 = band(lam[reg], 0)
        fdma_lu(l, d, u1, u2)
        xr = x[:, reg]
        fdma_solve(l, d, u1, u2, xr)
        x[:, reg] = xr
    if sing.any():
        l, d, u1, u2 = band(lam[sing], 1)
        fdma_lu(l, d, u1, u2)
        xs = x[1:, sing]
        fdma_solve(l, d, u1, u2, xs)
        x[1:, sing] = xs
        x[0, sing] = 0.0
    return x
