"""Chebyshev and Shen-Galerkin bases on the GPU.

Mirrors pypde/bases/chebyshev.py and pypde/bases/spectralbase.py: the same
classes, keys and method names.  Every transform runs along axis 0 of a 1-D or
2-D float64 CUDA tensor (numpy input is moved to the device) through the C ABI
in include/pgx.h.  Operator matrices (S, B, I) are host NumPy arrays built at
setup time, as in the reference.
"""
import ctypes

import numpy as np
import scipy.sparse
import torch

from . import _lib
from ._dev import empty_like_axis, geom, stream, to_dev
from .autodiff import linear
from .host import (dealias_size, gauss_lobatto, pseudoinverse_d2, stencil_matrix)


def Base(N, key, *args, **kwargs):
    """Base factory by key (spectralbase.py:12-45)."""
    return _bases_from_key(key)(N, *args, **kwargs)


def _bases_from_key(key):
    table = {"CH": Chebyshev, "Chebyshev": Chebyshev, "CD": ChebDirichlet, "ChebDirichlet": ChebDirichlet,
             "CN": ChebNeumann, "ChebNeumann": ChebNeumann, "DC": DirichletC, "DirichletC": DirichletC,
             "NC": NeumannC, "NeumannC": NeumannC}
    if key not in table:
        raise ValueError("Key {:} not available.".format(key))
    return table[key]


class MetaBase:
    """Common base (spectralbase.py:48-247): size, grid, dealiased twin, stencil."""

    def __init__(self, N, x, dealias=None):
        self._N = N
        self._x = x
        self.name = self.__class__.__name__
        self.id = None
        if dealias is not None:
            self.create_dealiased_base(self.N * dealias)

    @property
    def x(self):
        return self._x

    @property
    def N(self):
        """Number of grid points in physical space."""
        return self._N

    @property
    def M(self):
        """Number of coefficients without BC."""
        return len(range(*self.slice().indices(self.N)))

    def slice(self):
        return slice(0, self.N)

    def create_dealiased_base(self, size):
        self.dealias = self.__class__(int(size), dealias=None)

    @property
    def S(self):
        if not hasattr(self, "_S"):
            self._S = self.stencil() if hasattr(self, "stencil") else np.eye(self.N)
        return self._S

    @property
    def ST(self):
        return self.S.T

    @property
    def S_sp(self):
        return scipy.sparse.csc_matrix(self.S)

    @property
    def ST_sp(self):
        return scipy.sparse.csc_matrix(self.ST)


def _along0(f):
    f = to_dev(f)
    if f.dim() not in (1, 2):
        raise NotImplementedError("ndim must be less than 3")
    return f


class Chebyshev(MetaBase):
    """Chebyshev polynomials T_k on Gauss-Lobatto points (chebyshev.py:22-165)."""

    def __init__(self, N, dealias=None):
        MetaBase.__init__(self, N, gauss_lobatto(N - 1), dealias)
        self.id = "CH"
        self.family_id = "CH"

    _DCT_T = {_lib.DCT_FWD: _lib.DCT_FWD_T, _lib.DCT_BWD: _lib.DCT_BWD_T,
              _lib.DCT_FWD_T: _lib.DCT_FWD, _lib.DCT_BWD_T: _lib.DCT_BWD}

    def _dct_raw(self, f, mode, n_out):
        n_in = f.shape[0]
        if n_in > self.N or n_out > self.N:
            raise ValueError("input or output longer than the base")
        out = empty_like_axis(f, 0, n_out)
        p, s0, s1, _, nl = geom(f, 0)
        q, t0, t1, no, _ = geom(out, 0)
        _lib.check(_lib.lib().pgx_dct1(p, s0, s1, n_in, q, t0, t1, no, self.N, nl, 0, mode, stream()), "dct1")
        return out

    def _dct(self, f, mode, n_out=None):
        """DCT of mode ``mode`` along axis 0; input zero-padded and output truncated to n_out.

        Differentiable: the transpose is the transposed mode with the lengths swapped."""
        f = _along0(f)
        n_in, n_out = f.shape[0], self.N if n_out is None else n_out
        if mode == _lib.DCT_RAW:
            if f.requires_grad and torch.is_grad_enabled():
                raise NotImplementedError("dctn is not differentiable; use forward_fft / backward_fft")
            return self._dct_raw(f, mode, n_out)
        mt = self._DCT_T[mode]
        return linear(f, lambda x: self._dct_raw(x, mode, n_out), lambda g: self._dct_raw(g, mt, n_in))

    def forward_fft(self, f, mass=True):
        """Physical -> Chebyshev coefficients (chebyshev.py:67-76)."""
        c = self._dct(f, _lib.DCT_FWD)
        if not mass:  # undo the mass factor [1, 2, ..., 2, 1]
            c[1:-1] *= 0.5
        return c

    def backward_fft(self, c):
        """Chebyshev coefficients -> physical (chebyshev.py:78-83)."""
        return self._dct(c, _lib.DCT_BWD)

    def dctn(self, f, axes=(0,)):
        """Unnormalised DCT-I along axis 0 (chebyshev.py:85-93)."""
        if tuple(axes) != (0,):
            raise NotImplementedError("dctn acts along axis 0")
        return self._dct(f, _lib.DCT_RAW)

    def derivative(self, fhat, deriv, out_cheby=True):
        """Chebyshev recurrence applied ``deriv`` times (chebyshev.py:117-131)."""
        if deriv == 0:
            return fhat
        return linear(_along0(fhat), lambda x: self._diff(x, deriv, "pgx_cheb_diff"),
                      lambda g: self._diff(g, deriv, "pgx_cheb_diff_t"))

    @staticmethod
    def _diff(f, deriv, fn):
        out = empty_like_axis(f, 0, f.shape[0])
        p, s0, s1, n, nl = geom(f, 0)
        q, t0, t1, _, _ = geom(out, 0)
        _lib.check(getattr(_lib.lib(), fn)(p, s0, s1, q, t0, t1, n, nl, 0, deriv, stream()), fn)
        return out

    def solve_mass(self, f):
        f = to_dev(f)
        m = np.full(self.N, 2.0)
        m[0] = m[-1] = 1.0
        m = to_dev(m)
        return f * (m if f.dim() == 1 else m[:, None])

    def B(self, deriv, discardrow=0):
        """Pseudo-inverse of D^deriv (chebyshev.py:155-161)."""
        if deriv != 2:
            raise ValueError("deriv>2 not supported" if deriv > 2 else "only deriv == 2 is on this path")
        return pseudoinverse_d2(self.N)[discardrow:, :]

    def I(self, discardrow=0):  # noqa: E743
        return np.eye(self.N)[discardrow:, :]


class _StencilPlan:
    """Device tables of a ChebDirichlet / ChebNeumann stencil (pgx_stencil_plan)."""

    def __init__(self, key, N):
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().pgx_stencil_plan_create(key.encode(), N, ctypes.byref(h)), "stencil plan")
        self.h = h

    def __del__(self):
        try:
            _lib.lib().pgx_stencil_plan_destroy(self.h)
        except Exception:
            pass


class GalerkinChebyshev(MetaBase):
    """Composite Chebyshev space u = S v (chebyshev.py:168-363)."""

    _key = None

    def __init__(self, N, dealias=None):
        MetaBase.__init__(self, N, gauss_lobatto(N - 1), dealias)
        self._bc = None
        self.family_id = "CH"
        self.family = Chebyshev(self.N)

    def slice(self):
        return slice(0, self.N - 2)

    def stencil(self, transpose=False):
        S = stencil_matrix(self._key, self.N)
        return S.T if transpose else S

    @property
    def _plan(self):
        if not hasattr(self, "_splan"):
            self._splan = _StencilPlan(self._key, self.N)
        return self._splan

    def forward_fft(self, f, bc=None):
        """Physical -> Galerkin coefficients (chebyshev.py:241-266)."""
        f = to_dev(f)
        if bc is not None:
            f = f - self.eval_inhomogeneous(bc)
        return self.from_chebyshev(self.family.forward_fft(f))

    def backward_fft(self, c, bc=None):
        """Galerkin coefficients -> physical (chebyshev.py:268-285)."""
        u = self.to_chebyshev(c)
        if bc is not None:
            u = u + self.bc.to_chebyshev(bc)
        return self.family.backward_fft(u)

    def _stencil_op(self, x, fn, n_in, n_out):
        if x.shape[0] != n_in:
            raise ValueError("%s: expected %d points along the axis, got %d" % (fn, n_in, x.shape[0]))
        out = empty_like_axis(x, 0, n_out)
        p, s0, s1, _, nl = geom(x, 0)
        q, t0, t1, _, _ = geom(out, 0)
        _lib.check(getattr(_lib.lib(), fn)(self._plan.h, p, s0, s1, q, t0, t1, nl, 0, stream()), fn)
        return out

    def to_chebyshev(self, vhat):
        """u = S v (chebyshev.py:287-293); transpose S^T."""
        v = _along0(vhat)
        assert v.shape[0] == self.M, "{} {}".format(v.shape[0], self.M)
        return linear(v, lambda x: self._stencil_op(x, "pgx_stencil_to_chebyshev", self.M, self.N),
                      lambda g: self._stencil_op(g, "pgx_stencil_transpose", self.N, self.M))

    def from_chebyshev(self, uhat):
        """v = (S^T S)^-1 S^T u (chebyshev.py:295-337); transpose S (S^T S)^-1."""
        u = _along0(uhat)
        assert u.shape[0] == self.N, "Shape mismatch ({:3}) ({:3})".format(u.shape[0], self.N)
        return linear(u, lambda x: self._stencil_op(x, "pgx_stencil_from_chebyshev", self.N, self.M),
                      lambda g: self._stencil_op(g, "pgx_stencil_from_chebyshev_t", self.M, self.N))

    def eval_inhomogeneous(self, bchat):
        return self.bc.backward_fft(bchat)

    def derivative(self, vhat, deriv, out_cheby=True):
        """Derivative of Galerkin coefficients, Chebyshev output (chebyshev.py:347-363)."""
        duhat = self.family.derivative(self.to_chebyshev(vhat), deriv)
        if out_cheby:
            return duhat
        return self.from_chebyshev(duhat)


class ChebDirichlet(GalerkinChebyshev):
    """phi_k = T_k - T_{k+2} (chebyshev.py:366-392)."""

    _key = "CD"

    def __init__(self, N, dealias=None):
        GalerkinChebyshev.__init__(self, N, dealias)
        self.id = "CD"
        self.bc = DirichletC(N)


class ChebNeumann(GalerkinChebyshev):
    """phi_k = T_k - k^2/(k+2)^2 T_{k+2} (chebyshev.py:410-436)."""

    _key = "CN"

    def __init__(self, N, dealias=None):
        GalerkinChebyshev.__init__(self, N, dealias)
        self.id = "CN"
        self.bc = NeumannC(N)


class _BCBase(GalerkinChebyshev):
    """Two-mode boundary bases (chebyshev.py:538-597): tiny 2 x N operators applied
    as dense matrices through pgx_matrix_apply."""

    def slice(self):
        return slice(0, 2)

    def _matrix(self, name, A):
        if not hasattr(self, name):
            setattr(self, name, MatrixApply(A))
        return getattr(self, name)

    def to_chebyshev(self, vhat):
        v = _along0(vhat)
        assert v.shape[0] == 2
        return self._matrix("_to", self.stencil()).apply(v, 0)

    def from_chebyshev(self, c):
        """Solve S[:2,:2] x = c[:2] (chebyshev.py:564-566)."""
        A = np.zeros((2, self.N))
        A[:, :2] = np.linalg.inv(self.stencil()[:2, :2])
        return self._matrix("_from", A).apply(_along0(c), 0)


class DirichletC(_BCBase):
    _key = "DC"

    def __init__(self, N, dealias=None):
        GalerkinChebyshev.__init__(self, N, dealias)
        self.id = "DC"
        self.is_bc = True


class NeumannC(_BCBase):
    _key = "NC"

    def __init__(self, N, dealias=None):
        GalerkinChebyshev.__init__(self, N, dealias)
        self.id = "NC"
        self.is_bc = True


class MatrixApply:
    """A host matrix applied along an axis on the device (pgx_matrix_plan)."""

    def __init__(self, A):
        A = np.ascontiguousarray(np.real(A), dtype=np.float64)
        self.rows, self.cols = A.shape
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().pgx_matrix_plan_create(A.ctypes.data_as(ctypes.c_void_p), self.rows, self.cols,
                                                      ctypes.byref(h)), "matrix plan")
        self.h = h
        self.banded = bool(_lib.lib().pgx_matrix_plan_is_banded(h))
        self._A = A
        self._T = None

    @property
    def T(self):
        """The transposed operator (its own device plan, built on first use)."""
        if self._T is None:
            self._T = MatrixApply(self._A.T)
            self._T._T = self
        return self._T

    def apply(self, b, axis):
        """out = A b along ``axis``; differentiable (transpose A^T)."""
        b = to_dev(b)
        if b.shape[axis] != self.cols:
            raise ValueError("Shape mismatch: N {:4d} | b.shape[axis] {:4d}".format(self.cols, b.shape[axis]))
        return linear(b, lambda x: self._apply(x, axis), lambda g: self.T._apply(g, axis))

    def _apply(self, b, axis):
        if b.shape[axis] != self.cols:
            raise ValueError("Shape mismatch: N {:4d} | b.shape[axis] {:4d}".format(self.cols, b.shape[axis]))
        out = empty_like_axis(b, axis, self.rows)
        p, s0, s1, _, nl = geom(b, axis)
        q, t0, t1, _, _ = geom(out, axis)
        _lib.check(_lib.lib().pgx_matrix_apply(self.h, p, s0, s1, q, t0, t1, nl, axis, stream()), "matrix apply")
        return out

    def __del__(self):
        try:
            _lib.lib().pgx_matrix_plan_destroy(self.h)
        except Exception:
            pass


__all__ = ["Base", "MetaBase", "Chebyshev", "GalerkinChebyshev", "ChebDirichlet", "ChebNeumann",
           "DirichletC", "NeumannC", "MatrixApply", "dealias_size"]
