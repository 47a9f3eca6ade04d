"""Fields in physical and spectral space on the GPU (pypde/field.py).

``v`` and ``vhat`` are float64 CUDA tensors; assigning a NumPy array moves it
to the device.  ``write`` / ``read`` keep the reference's snapshot layout
(``io.py``); plotting is not provided.
"""
import numpy as np
import torch

from . import _lib
from ._dev import to_dev, DTYPE, device
from .bases import MetaBase
from .spectralspace import SpectralSpace, SpectralSpaceBC


def zero_pad(array, target_length, axis=0):
    """zero_pad (bases/utils.py:88-109) for device tensors."""
    pad = target_length - array.shape[axis]
    if pad <= 0:
        return array
    shape = list(array.shape)
    shape[axis] = target_length
    out = torch.zeros(shape, dtype=DTYPE, device=array.device)
    out.narrow(axis, 0, array.shape[axis]).copy_(array)
    return out


def zero_unpad(array, target_length, axis=0):
    return array.narrow(axis, 0, target_length)


def _on_axis(t, axis, fn):
    """``fn`` (a 1-D operator along axis 0) applied along ``axis`` of ``t`` through a transposed
    view: the C ABI takes strides, so nothing is copied."""
    return fn(t) if axis == 0 else fn(t.transpose(axis, 0)).transpose(axis, 0)


def _values(coef_base, grid_base, c):
    """Coefficient lines of ``coef_base`` -> values on ``grid_base``'s points (axis 0).  A shorter
    coefficient base (the undealiased one) is not padded by a copy: the stencil maps its own
    coefficients to Chebyshev ones, and the backward DCT of the grid's length reads those and
    zero-fills the rest of the line (the kernel's input length, like the fused passes' SETLEN).
    Zero-padding commutes with the Shen stencils, whose entries depend on the row index only."""
    u = coef_base.to_chebyshev(c) if hasattr(coef_base, "to_chebyshev") else _as_lines(c)
    fam = getattr(grid_base, "family", grid_base)
    return fam._dct(u, _lib.DCT_BWD)


def _as_lines(t):
    if t.dim() not in (1, 2):
        raise NotImplementedError("ndim must be less than 3")
    return t


class FieldBase:
    """Transforms shared by Field and FieldBC (field.py:9-56).

    Axis 0 then axis 1, each one strided C-ABI pass over a view.  A 3/2-dealiased field keeps
    its undealiased twin's bases (``_coef_bases``): a backward transform reads coefficients of
    either length (the short ones are zero-filled inside the DCT, no padded copy), a forward one
    returns the leading coefficients of the long transform as a view (the truncation)."""

    def _coef_base(self, axis, n):
        grid = self.xs[axis]
        if n == grid.M:
            return grid
        short = getattr(self, "_coef_bases", None)
        if short is not None and n == short[axis].M:
            return short[axis]
        raise ValueError("axis %d: %d coefficients, the field has %d%s" % (
            axis, n, grid.M, "" if short is None else " or %d" % short[axis].M))

    def backward(self, vhat=None, dealias_before=None):
        data = self.vhat if vhat is None else to_dev(vhat)
        pad = self.dealiased_space if dealias_before is None else dealias_before
        for axis, grid in enumerate(self.xs):
            n = data.shape[axis]
            coef = self._coef_base(axis, n) if (pad or n != grid.M) else grid
            data = _on_axis(data, axis, lambda t, c=coef, g=grid: _values(c, g, t))
        if vhat is not None:
            return data
        self.v = data

    def forward(self, v=None, undealias_after=None):
        data = self.v if v is None else to_dev(v)
        cut = self.dealiased_space if undealias_after is None else undealias_after
        keep = self.size_undealiased if cut else [b.M for b in self.xs]
        for axis in range(self.ndim):
            data = self.forward_fft(data, axis=axis).narrow(axis, 0, keep[axis])
        if v is not None:
            return data
        self.vhat = data

    @property
    def v(self):
        return self._v

    @v.setter
    def v(self, value):
        self._v = to_dev(value)

    @property
    def vhat(self):
        return self._vhat

    @vhat.setter
    def vhat(self, value):
        self._vhat = to_dev(value)

    @property
    def x(self):
        return self.xs[0].x

    @property
    def y(self):
        if self.ndim < 2:
            raise ValueError("Dimension y not defined for ndim<2.")
        return self.xs[1].x

    @staticmethod
    def _cell_widths(x):
        xm = np.zeros(x.size + 1)
        xm[0], xm[-1] = x[0], x[-1]
        xm[1:-1] = (x[1:] + x[:-1]) / 2.0
        return np.diff(xm)

    @property
    def dx(self):
        return self._cell_widths(self.x)

    @property
    def dy(self):
        return self._cell_widths(self.y)


class Field(SpectralSpace, FieldBase):
    """Field with physical values ``v`` and coefficients ``vhat`` (field.py:180-356)."""

    def __init__(self, bases):
        if isinstance(bases, MetaBase):
            bases = [bases]
        SpectralSpace.__init__(self, bases)
        self.bases = bases
        device()
        self.v = np.zeros(self.shape_physical)
        self.vhat = np.zeros(self.shape_spectral)
        self.field_bc = None
        self.t = 0
        self._history = []
        self.dealiased_space = False
        self.create_dealiased_field(bases)

    def create_dealiased_field(self, bases):
        """The 3/2-grid twin (field.py:271-276): its own bases are the dealiased ones; it reads and
        returns coefficients of this field's size."""
        if not all(hasattr(b, "dealias") for b in bases):
            return
        twin = Field([b.dealias for b in bases])
        twin._coef_bases = list(self.xs)
        twin.size_undealiased = list(self.shape_spectral)
        twin.dealiased_space = True
        self.dealias = twin

    def add_field_bc(self, field_bc):
        if not isinstance(field_bc, FieldBC):
            raise AssertionError("add_field_bc expects a FieldBC")
        self.field_bc = field_bc

    # the field splits into the part that meets homogeneous conditions (v) and the lift that
    # carries the boundary values (the FieldBC's v); without a lift the latter is zero
    @property
    def inhomogeneous(self):
        return 0 if self.field_bc is None else self.field_bc.v

    @property
    def homogeneous(self):
        return self.v

    @property
    def total(self):
        lift = self.inhomogeneous
        return self.v if isinstance(lift, int) else torch.add(self.v, lift)

    def make_homogeneous(self):
        """v minus the lift (field.py:286-291); warns when no FieldBC was added."""
        if self.field_bc is None:
            import warnings
            warnings.warn("No inhomogeneous field found. Call add_bc(bchat,axis) first!")
            return self.v
        return torch.sub(self.v, self.field_bc.v)

    # time history kept by save(): (time, device copy of v) pairs; V and T are their columns
    @property
    def V(self):
        return [v for _, v in self._history]

    @property
    def T(self):
        return [t for t, _ in self._history]

    def save(self, transform=True):
        """Append (t, v) to the history (field.py:323-330); v is brought up to date first unless
        ``transform`` is False."""
        if transform:
            self.backward()
        self._history.append((self.t, self.v.clone()))

    def write(self, filename="file_0.h5", dict=None, leading_str="flow", add_time=True,  # noqa: A002
              grp_name=""):
        """field.py:83-117: v, vhat, time, x, y (and ``dict``) into the snapshot file."""
        from . import io
        with io.Store(io.snapshot_name(self.t, filename, leading_str, add_time), "a") as st:
            io.write_field(self, st, grp_name, dict)

    def read(self, filename="file_0.h5", dict=None, leading_str="flow", add_time=True,  # noqa: A002
             grp_name=""):
        """field.py:137-173: v, vhat, time (and the ``dict`` keys, filled in place)."""
        from . import io
        with io.Store(io.snapshot_name(self.t, filename, leading_str, add_time), "r") as st:
            io.read_field(self, st, grp_name, dict)


class FieldBC(SpectralSpaceBC, FieldBase):
    """Inhomogeneous boundary-condition field (field.py:359-414)."""

    def __init__(self, bases, axis):
        SpectralSpaceBC.__init__(self, bases, axis)
        self.v = np.zeros(self.shape_physical)
        self.vhat = np.zeros(self.shape_spectral)
        self.dealiased_space = False

    def add_bc(self, bc):
        """``bc`` is forward transformed along self.axis only; other axes physical."""
        expected = list(self.shape_physical)
        expected[self.axis] = self.shape_spectral[self.axis]
        assert tuple(bc.shape) == tuple(expected)
        self.v = self.backward_fft(to_dev(bc), axis=self.axis)
        self.forward()


class MultiField:
    """Fields stepped and saved together under group names (field.py:417-465)."""

    def __init__(self, fields, names):
        bad = [type(f).__name__ for f in fields if not isinstance(f, Field)]
        if bad:
            raise ValueError("Must be of type Field.")
        self._by_name = dict(zip(names, fields))

    @property
    def fields(self):
        return list(self._by_name.values())

    @property
    def names(self):
        return list(self._by_name)

    def save(self):
        for f in self._by_name.values():
            f.save()

    def write(self, filename=None, leading_str="", add_time=True, dict={}):  # noqa: A002, B006
        """field.py:450-459: every field in its group of one snapshot file."""
        from . import io
        name = io.snapshot_name(self.fields[0].t, filename, leading_str, add_time)
        with io.Store(name, "a") as st:
            for f, n in zip(self.fields, self.names):
                io.write_field(f, st, n, dict)
        return io.container_path(name)

    def read(self, filename=None, leading_str="", add_time=True, dict={}):  # noqa: A002, B006
        """field.py:440-448."""
        from . import io
        name = io.snapshot_name(self.fields[0].t, filename, leading_str, add_time)
        with io.Store(name, "r") as st:
            for f, n in zip(self.fields, self.names):
                io.read_field(f, st, n, dict)

    def update_time(self, dt):
        """Advance every field's clock by dt (field.py:462-465)."""
        for f in self._by_name.values():
            f.t += dt
