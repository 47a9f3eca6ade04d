"""2-D fields, transforms with 3/2 dealiasing and field operations (oracle, test infrastructure).

Reference: pypde/field.py, pypde/field_operations.py, pypde/bases/utils.py,
pypde/bases/spectralspace.py.  A 2-D space is a pair of basis keys plus the
physical sizes (N along x = axis 0, M along y = axis 1).
"""
import numpy as np

from . import spectral as sp


def zero_pad(a, target, axis):
    """zero_pad (bases/utils.py:88-109)."""
    pad = target - a.shape[axis]
    if pad <= 0:
        return a
    w = [(0, 0)] * a.ndim
    w[axis] = (0, pad)
    return np.pad(a, w)


def zero_unpad(a, target, axis):
    """zero_unpad (bases/utils.py:112-115)."""
    sl = [slice(None)] * a.ndim
    sl[axis] = slice(0, target)
    return a[tuple(sl)]


class Space2D:
    """Field / FieldBC space: bases ``keys`` on physical shape ``shape``.

    ``dealias`` mirrors Field.create_dealiased_field (field.py:271-276): the
    dealiased twin has bases of size int(1.5 N) and remembers the
    un-dealiased coefficient counts for the unpad after each forward axis.
    """

    def __init__(self, keys, shape):
        self.keys = tuple(sp.canon(k) for k in keys)
        self.shape = tuple(shape)
        self.M = tuple(sp.n_coeffs(k, n) for k, n in zip(self.keys, self.shape))

    @property
    def dealias(self):
        d = Space2D(self.keys, tuple(sp.dealias_size(n) for n in self.shape))
        d.undealiased_M = self.M
        return d

    def x(self, axis=0):
        return sp.gauss_lobatto(self.shape[axis] - 1)

    # FieldBase.forward / backward (field.py:14-56)
    def forward(self, v, undealias=False):
        vhat = v
        for axis in range(2):
            vhat = sp.forward(self.keys[axis], vhat, axis)
            if undealias:
                vhat = zero_unpad(vhat, self.undealiased_M[axis], axis)
        return vhat

    def backward(self, vhat, dealias=False):
        v = vhat
        for axis in range(2):
            if dealias:
                v = zero_pad(v, self.M[axis], axis)
            v = sp.backward(self.keys[axis], v, axis, N=self.shape[axis])
        return v

    def dealias_forward(self, v):
        """``field.dealias.forward(v)`` for a field built with dealias=3/2."""
        return self.dealias.forward(v, undealias=True)

    def dealias_backward(self, vhat):
        """``field.dealias.backward(vhat)`` for a field built with dealias=3/2."""
        return self.dealias.backward(vhat, dealias=True)

    def derivative(self, vhat, deriv, axis):
        """SpectralSpace.derivative (spectralspace.py:54-60), Chebyshev output."""
        return sp.derivative(self.keys[axis], vhat, deriv, axis, N=self.shape[axis])

    # FieldBase.dx / dy (field.py:68-80)
    def cell_widths(self, axis):
        x = self.x(axis)
        xm = np.zeros(x.size + 1)
        xm[0], xm[-1] = x[0], x[-1]
        xm[1:-1] = (x[1:] + x[:-1]) / 2.0
        return np.diff(xm)


def grad(space, vhat, deriv, scale=None):
    """grad (field_operations.py:8-56): Chebyshev coefficients of the derivative."""
    dv = vhat
    for axis in range(2):
        dv = space.derivative(dv, deriv[axis], axis)
        if scale is not None:
            dv = dv / scale[axis] ** deriv[axis]
    return dv


def galerkin_to_cheby(space, vhat):
    """galerkin_to_cheby (field_operations.py:71-80)."""
    for axis in range(2):
        k = space.keys[axis]
        if k in (sp.CD, sp.CN):
            vhat = sp.to_chebyshev(k, vhat, axis)
        elif k in (sp.DC, sp.NC):
            vhat = sp.to_chebyshev_bc(k, vhat, space.shape[axis], axis)
    return vhat


def cheby_to_galerkin(space, uhat):
    """cheby_to_galerkin (field_operations.py:59-68)."""
    for axis in range(2):
        if space.keys[axis] != sp.CH:
            uhat = sp.from_chebyshev(space.keys[axis], uhat, axis)
    return uhat


def conv_term(space, vhat, u, deriv, deriv_space, dealias, scale):
    """conv_term (field_operations.py:83-129): u * d(v)/d(deriv) in physical space."""
    dv = grad(space, vhat, deriv, scale)
    if dealias:
        return deriv_space.dealias_backward(dv) * u
    return deriv_space.backward(dv) * u


def convective_term(space, vhat, ux, uz, deriv_space, add_bc=None, dealias=False, scale=None):
    """convective_term (field_operations.py:132-169): F[ux dv/dx + uz dv/dz (+ add_bc)]."""
    conv = conv_term(space, vhat, ux, (1, 0), deriv_space, dealias, scale)
    conv = conv + conv_term(space, vhat, uz, (0, 1), deriv_space, dealias, scale)
    if add_bc is not None:
        conv = conv + add_bc
    if dealias:
        return deriv_space.dealias_forward(conv)
    return deriv_space.forward(conv)


def avg_x(f, dx):
    """avg_x (field_operations.py:175-176)."""
    return np.sum(f * dx[:, None], axis=0) / np.sum(dx)


def avg_vol(f, dx, dy):
    """avg_vol (field_operations.py:179-181)."""
    favgx = np.sum(f * dx[:, None], axis=0) / np.sum(dx)
    return np.sum(favgx * dy) / np.sum(dy)
