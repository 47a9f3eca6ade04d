"""Field operations on the GPU (pypde/field_operations.py)."""
import numpy as np
import torch

from ._dev import to_dev
from .bases import Base
from .field import Field, FieldBC


def grad(field, deriv, return_field=False, scale=None):
    """Chebyshev coefficients of a derivative of ``field.vhat`` (field_operations.py:8-56)."""
    assert isinstance(field, (Field, FieldBC))
    if isinstance(deriv, int):
        deriv = (deriv,)
    assert field.ndim == len(deriv)
    dvhat = field.vhat
    for axis in range(field.ndim):
        dvhat = field.derivative(dvhat, deriv[axis], axis=axis)
        if scale is not None and deriv[axis] != 0:
            assert len(scale) == field.ndim
            dvhat = dvhat / scale[axis] ** deriv[axis]
    if return_field:
        xs = [f.family if hasattr(f, "family") else f for f in field.xs]
        out = Field(xs)
        out.vhat = dvhat
        return out
    return dvhat


def cheby_to_galerkin(uhat, galerkin_field):
    """from_chebyshev along every axis with a stencil (field_operations.py:59-68)."""
    uhat = to_dev(uhat)
    for axis in range(uhat.dim()):
        b = galerkin_field.xs[axis]
        if hasattr(b, "from_chebyshev"):
            if axis == 0:
                uhat = b.from_chebyshev(uhat)
            else:
                uhat = b.from_chebyshev(uhat.transpose(0, axis)).transpose(0, axis)
    return uhat


def galerkin_to_cheby(vhat, galerkin_field):
    """to_chebyshev along every axis with a stencil (field_operations.py:71-80)."""
    vhat = to_dev(vhat)
    for axis in range(vhat.dim()):
        b = galerkin_field.xs[axis]
        if hasattr(b, "to_chebyshev"):
            if axis == 0:
                vhat = b.to_chebyshev(vhat)
            else:
                vhat = b.to_chebyshev(vhat.transpose(0, axis)).transpose(0, axis)
    return vhat


def _deriv_field(v_field, dealias):
    d = 3 / 2 if dealias else None
    return Field([Base(v_field.shape[0], "CH", dealias=d), Base(v_field.shape[1], "CH", dealias=d)])


def conv_term(v_field, u, deriv, deriv_field=None, dealias=False, scale=None):
    """u * dv/dx_i in physical space (field_operations.py:83-129)."""
    assert isinstance(v_field, Field), "v_field must be instance Field"
    if deriv_field is None:
        deriv_field = _deriv_field(v_field, dealias)
    vhat = grad(v_field, deriv, return_field=False, scale=scale)
    dvdx = deriv_field.dealias.backward(vhat) if dealias else deriv_field.backward(vhat)
    return dvdx * to_dev(u)


def convective_term(v_field, ux, uz, deriv_field=None, add_bc=None, dealias=False, scale=None):
    """Spectral coefficients of ux dv/dx + uz dv/dz (+ add_bc) (field_operations.py:132-169)."""
    if deriv_field is None:
        deriv_field = _deriv_field(v_field, dealias)
    conv = conv_term(v_field, ux, (1, 0), deriv_field, dealias, scale=scale)
    conv = conv + conv_term(v_field, uz, (0, 1), deriv_field, dealias, scale=scale)
    if add_bc is not None:
        conv = conv + to_dev(add_bc)
    if dealias:
        return deriv_field.dealias.forward(conv)
    return deriv_field.forward(conv)


def avg_x(f, dx):
    """Cell-width weighted mean over x (field_operations.py:175-176)."""
    f = to_dev(f)
    dx = to_dev(np.asarray(dx))
    return (f * dx[:, None]).sum(dim=0) / dx.sum()


def avg_vol(f, dx, dy):
    """Cell-width weighted volume mean (field_operations.py:179-181)."""
    dy = to_dev(np.asarray(dy))
    return (avg_x(f, dx) * dy).sum() / dy.sum()


def interpolate(Field_old, Field_new, spectral=True):
    """Copy the overlapping block of coefficients (or values) (field_operations.py:184-220)."""
    old = Field_old.vhat if spectral else Field_old.v
    new = Field_new.vhat if spectral else Field_new.v
    if old.dim() != new.dim():
        raise ValueError("Field must be of same dimension!")
    buf = torch.zeros([max(i, j) for i, j in zip(old.shape, new.shape)], dtype=old.dtype, device=old.device)
    buf[tuple(slice(0, n) for n in old.shape)] = old
    new.copy_(buf[tuple(slice(0, n) for n in new.shape)])
    if spectral:
        Field_new.backward()
    else:
        Field_new.forward()
