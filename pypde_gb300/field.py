"""Fields in physical and spectral space on the GPU (pypde/field.py).

``v`` and ``vhat`` are float64 CUDA tensors; assigning a NumPy array moves it
to the device.  ``write`` / ``read`` keep the reference's snapshot layout
(``io.py``); plotting is not provided.
"""
import numpy as np
import torch

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


class FieldBase:
    """Transforms shared by Field and FieldBC (field.py:9-56)."""

    def forward(self, v=None, undealias_after=None):
        vhat = self.v if v is None else to_dev(v)
        if undealias_after is None:
            undealias_after = self.dealiased_space
        for axis in range(self.ndim):
            vhat = self.forward_fft(vhat, axis=axis)
            if undealias_after:
                vhat = zero_unpad(vhat, self.size_undealiased[axis], axis=axis)
        if v is None:
            self.vhat = vhat
        else:
            return vhat

    def backward(self, vhat=None, dealias_before=None):
        v = self.vhat if vhat is None else to_dev(vhat)
        if dealias_before is None:
            dealias_before = self.dealiased_space
        for axis in range(self.ndim):
            if dealias_before:
                v = zero_pad(v, self.xs[axis].M, axis=axis)
            v = self.backward_fft(v, axis=axis)
        if vhat is None:
            self.v = v
        else:
            return v

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
        self.V = []
        self.T = []
        self.dealiased_space = False
        self.create_dealiased_field(bases)

    def create_dealiased_field(self, bases):
        if all(hasattr(i, "dealias") for i in bases):
            self.dealias = Field([i.dealias for i in bases])
            self.dealias.size_undealiased = [self.xs[i].M for i in range(self.ndim)]
            self.dealias.dealiased_space = True

    def add_field_bc(self, field_bc):
        assert isinstance(field_bc, FieldBC)
        self.field_bc = field_bc

    def make_homogeneous(self):
        if self.field_bc is None:
            import warnings
            warnings.warn("No inhomogeneous field found. Call add_bc(bchat,axis) first!")
        return self.v - self.inhomogeneous

    @property
    def total(self):
        return self.homogeneous + self.inhomogeneous

    @property
    def homogeneous(self):
        return self.v

    @property
    def inhomogeneous(self):
        if self.field_bc is not None:
            return self.field_bc.v
        return 0

    def save(self, transform=True):
        if transform:
            self.backward()
        self.V.append(self.v.clone())
        self.T.append(self.t)

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
    """Collection of fields updated together (field.py:417-465)."""

    def __init__(self, fields, names):
        self.fields, self.names = [], []
        for f, n in zip(fields, names):
            if not isinstance(f, Field):
                raise ValueError("Must be of type Field.")
            self.fields.append(f)
            self.names.append(n)

    def save(self):
        for f in self.fields:
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
        for f in self.fields:
            f.t += dt
