"""Chebyshev / Shen-Galerkin bases restated in NumPy (oracle, test infrastructure).

Reference: pypde/bases/chebyshev.py, pypde/bases/dmsuite.py,
pypde/bases/fortran/differentiate_cheby.f90, pypde/bases/spectralbase.py.
All arrays are float64; 1-D operations act along ``axis`` of an N-D array.
"""
import numpy as np
import scipy.fft

from . import _ck

from . import linalg

# Basis keys as accepted by pypde's Base() factory (spectralbase.py:25-45).
CH, CD, CN, DC, NC = "CH", "CD", "CN", "DC", "NC"
_KEYS = {"CH": CH, "Chebyshev": CH, "CD": CD, "ChebDirichlet": CD,
         "CN": CN, "ChebNeumann": CN, "DC": DC, "DirichletC": DC,
         "NC": NC, "NeumannC": NC}


def canon(key):
    if key not in _KEYS:
        raise ValueError("Key {:} not available.".format(key))
    return _KEYS[key]


def gauss_lobatto(n):
    """Gauss-Lobatto points for ``n`` intervals, ascending -1..1 (dmsuite.py:209-214)."""
    k = np.linspace(n, 0, n + 1)
    return np.sin(np.pi * (n - 2 * k) / (2 * n))


def dealias_size(N, factor=1.5):
    """Size of the dealiased sub-base: int(N*3/2) (spectralbase.py:77-78,94-96)."""
    return int(N * factor)


def n_coeffs(key, N):
    """Number of spectral coefficients M (spectralbase.py:89-92, chebyshev.py:208-213,561-562)."""
    key = canon(key)
    if key == CH:
        return N
    if key in (CD, CN):
        return N - 2
    return 2


# --------------------------------------------------------------------------
# DCT-I (chebyshev.py:85-93: scipy.fftpack.dctn(f, type=1, axes=(0,)))
# --------------------------------------------------------------------------
def dct1(f, axis=0):
    """Unnormalised DCT-I along ``axis``.

    y_k = x_0 + (-1)^k x_{n-1} + 2 sum_{j=1}^{n-2} x_j cos(pi j k / (n-1)).
    scipy.fft.dct(type=1) is bit-identical to the scipy.fftpack.dctn call the
    reference makes (both are pocketfft).
    """
    return scipy.fft.dct(np.asarray(f, dtype=np.float64), type=1, axis=axis)


def dct1_direct(f, axis=0):
    """O(n^2) cosine-sum DCT-I, the closed-form definition (for small n)."""
    f = np.moveaxis(np.asarray(f, dtype=np.float64), axis, 0)
    n = f.shape[0]
    j = np.arange(n)
    C = 2.0 * np.cos(np.pi * np.outer(j, j) / (n - 1))
    C[:, 0] = 1.0
    C[:, -1] = (-1.0) ** j
    return np.moveaxis(np.tensordot(C, f, axes=(1, 0)), 0, axis)


def _along(a, axis, vec):
    shape = [1] * a.ndim
    shape[axis] = -1
    return vec.reshape(shape)


def cheb_forward(f, axis=0, mass=True):
    """Chebyshev.forward_fft (chebyshev.py:67-76) + solve_mass (143-149)."""
    N = f.shape[axis]
    sign = (-1.0) ** np.arange(N)
    c = 0.5 * dct1(f, axis) / (N - 1)
    c = _along(c, axis, sign) * c
    if mass:
        m = np.full(N, 2.0)
        m[0] = m[-1] = 1.0
        c = _along(c, axis, m) * c
    return c


def cheb_backward(c, axis=0):
    """Chebyshev.backward_fft (chebyshev.py:78-83)."""
    N = c.shape[axis]
    sign = (-1.0) ** np.arange(N)
    sign[0] *= 2.0
    sign[-1] *= 2.0
    return 0.5 * dct1(_along(c, axis, sign) * c, axis)


# --------------------------------------------------------------------------
# Stencils S (N x M): Galerkin -> Chebyshev  (chebyshev.py:382-392, 426-436,
# 555-559, 586-590)
# --------------------------------------------------------------------------
def stencil(key, N):
    key = canon(key)
    if key == CH:
        return np.eye(N)
    M = n_coeffs(key, N)
    S = np.zeros((N, M))
    if key == CD:
        for i in range(M):
            S[i, i], S[i + 2, i] = 1.0, -1.0
    elif key == CN:
        for i in range(M):
            S[i, i], S[i + 2, i] = 1.0, -((i / (i + 2)) ** 2)
    elif key == DC:
        S[0, 0], S[1, 0] = 0.5, -0.5
        S[0, 1], S[1, 1] = 0.5, 0.5
    elif key == NC:
        S[0, 0], S[1, 0] = 0.5, -1.0 / 8.0
        S[0, 1], S[1, 1] = 0.5, 1.0 / 8.0
    return S


def _apply(A, v, axis):
    """Dense matrix along ``axis``: MatrixBase.dot_matrix (pypde/solver/matrix.py:48-53)."""
    v = np.moveaxis(v, axis, 0)
    return np.moveaxis(np.tensordot(A, v, axes=(1, 0)), 0, axis)


def to_chebyshev(key, v, axis=0):
    """GalerkinChebyshev.to_chebyshev: u = S v (chebyshev.py:287-293)."""
    key = canon(key)
    if key == CH:
        return v
    N = v.shape[axis] + 2 if key in (CD, CN) else None
    if key in (DC, NC):
        raise ValueError("bc bases need N; use to_chebyshev_bc")
    return _apply(stencil(key, N), v, axis)


def to_chebyshev_bc(key, v, N, axis=0):
    """to_chebyshev for the 2-mode boundary bases DirichletC / NeumannC."""
    return _apply(stencil(key, N), v, axis)


def stencil_inv_diags(key, N):
    """Diagonals -2, 0, +2 of S^T S (chebyshev.py:331-337)."""
    S = stencil(key, N)
    A = S.T @ S
    return np.diag(A, -2).copy(), np.diag(A, 0).copy(), np.diag(A, 2).copy()


def from_chebyshev(key, u, axis=0):
    """GalerkinChebyshev.from_chebyshev: v = (S^T S)^-1 S^T u (chebyshev.py:295-329).

    The least-squares system is solved by the offset-2 TDMA (tdma.f90:56-107);
    DirichletC / NeumannC solve a 2x2 system on modes 0,1 (chebyshev.py:564-566,595-597).
    """
    key = canon(key)
    if key == CH:
        return u
    N = u.shape[axis]
    if key in (DC, NC):
        S = stencil(key, N)
        um = np.moveaxis(u, axis, 0)[:2]
        return np.moveaxis(np.linalg.solve(S[:2, :2], um.reshape(2, -1)).reshape(um.shape), 0, axis)
    S = stencil(key, N)
    l2, d, u2 = stencil_inv_diags(key, N)
    rhs = _apply(S.T, u, axis)
    rhs = np.moveaxis(rhs, axis, 0)
    x = linalg.tdma_offset(l2, d, u2, rhs, 2)
    return np.moveaxis(x, 0, axis)


# --------------------------------------------------------------------------
# Derivative recurrence (differentiate_cheby.f90:28-53; chebyshev.py:117-131)
# --------------------------------------------------------------------------
def cheb_diff1(c, axis=0):
    """One Chebyshev derivative of coefficients along ``axis``.

    dc_{n-2} = 2(n-1) c_{n-1};  dc_j = dc_{j+2} + 2(j+1) c_{j+1}, j = n-3..1;
    dc_0 = dc_2/2 + c_1;  dc_{n-1} = 0 (f2py zero-fills the hidden output).
    """
    c = np.moveaxis(np.asarray(c, dtype=np.float64), axis, 0)
    n = c.shape[0]
    L = _ck.lib()
    if L is not None and n >= 3:
        cc = _ck.c64(c.reshape(n, -1))
        dc = np.zeros_like(cc)
        L.ok_cheb_diff1(_ck.ptr(cc), _ck.ptr(dc), n, cc.shape[1])
        return np.moveaxis(dc.reshape(c.shape), 0, axis)
    dc = np.zeros_like(c)
    dc[n - 2] = 2.0 * (n - 1) * c[n - 1]
    for j in range(n - 3, 0, -1):
        dc[j] = dc[j + 2] + 2.0 * (j + 1) * c[j + 1]
    dc[0] = dc[2] / 2.0 + c[1]
    return np.moveaxis(dc, 0, axis)


def cheb_diff(c, deriv, axis=0):
    """Chebyshev.derivative: apply the recurrence ``deriv`` times."""
    for _ in range(deriv):
        c = cheb_diff1(c, axis)
    return c


def derivative(key, v, deriv, axis=0, N=None):
    """Base derivative in Chebyshev output (chebyshev.py:117-131, 347-363).

    Galerkin input goes through S first, even when deriv == 0.
    """
    key = canon(key)
    if key == CH:
        return cheb_diff(v, deriv, axis) if deriv else v
    if key in (DC, NC):
        return cheb_diff(to_chebyshev_bc(key, v, N, axis), deriv, axis)
    return cheb_diff(to_chebyshev(key, v, axis), deriv, axis)


# --------------------------------------------------------------------------
# Galerkin transforms (chebyshev.py:241-285)
# --------------------------------------------------------------------------
def forward(key, f, axis=0):
    """Base forward_fft: physical -> spectral coefficients of ``key``."""
    key = canon(key)
    c = cheb_forward(f, axis)
    return c if key == CH else from_chebyshev(key, c, axis)


def backward(key, v, axis=0, N=None):
    """Base backward_fft: spectral coefficients of ``key`` -> physical."""
    key = canon(key)
    if key == CH:
        return cheb_backward(v, axis)
    if key in (DC, NC):
        return cheb_backward(to_chebyshev_bc(key, v, N, axis), axis)
    return cheb_backward(to_chebyshev(key, v, axis), axis)


# --------------------------------------------------------------------------
# Pseudo-inverse of D^2 (dmsuite.py:327-368; pinv.py:274-297; chebyshev.py:155-165)
# --------------------------------------------------------------------------
def pseudoinverse_d2(N):
    """N x N banded pseudo-inverse of the Chebyshev D^2 (diagonals -2, 0, +2)."""
    diag0 = np.zeros(N)
    diag0[2:-2] = [-1.0 / (2 * (i ** 2 - 1)) for i in range(2, N - 2)]
    diag1 = np.zeros(N - 2)
    diag1[2:-2] = [1.0 / (4 * i * (i + 1)) for i in range(2, N - 4)]
    diag2 = np.array([1.0 / (4 * i * (i - 1)) for i in range(2, N)])
    diag2[0] *= 2
    P = np.diag(diag0) + np.diag(diag1, 2) + np.diag(diag2, -2)
    P[np.abs(P) < 1e-12] = 0.0  # pinv.py:289 tosparse(tol=1e-12)
    return P


def B2(N):
    """Chebyshev.B(2, discardrow=2): rows 2: of the D^2 pseudo-inverse, (N-2) x N."""
    return pseudoinverse_d2(N)[2:, :]


def I2(N):
    """Chebyshev.I(discardrow=2): rows 2: of the identity, (N-2) x N."""
    return np.eye(N)[2:, :]
