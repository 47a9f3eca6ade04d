"""N-D spectral spaces (pypde/bases/spectralspace.py).

A 1-D basis op along ``axis`` is applied to a transposed view (zero-copy: the
C ABI takes strides), matching the reference's swapaxes pattern.
"""
from .bases import MetaBase


class SpectralSpace:
    """Collection of bases, one per axis (spectralspace.py:4-66)."""

    def __init__(self, bases):
        if isinstance(bases, MetaBase):
            bases = [bases]
        self._set_bases(bases)
        self.ndim = len(self.shape_physical)
        self.shape = self.shape_physical

    def _set_bases(self, bases):
        self.xs = list(bases)
        self.shape_physical = tuple(b.N for b in self.xs)
        self.shape_spectral = tuple(b.M for b in self.xs)

    def forward_fft(self, v, axis):
        if axis == 0:
            return self.xs[axis].forward_fft(v)
        return self.xs[axis].forward_fft(v.transpose(axis, 0)).transpose(axis, 0)

    def backward_fft(self, vhat, axis):
        if axis == 0:
            return self.xs[axis].backward_fft(vhat)
        return self.xs[axis].backward_fft(vhat.transpose(axis, 0)).transpose(axis, 0)

    def derivative(self, vhat, deriv, axis, out_cheby=True):
        if axis == 0:
            return self.xs[axis].derivative(vhat, deriv, out_cheby)
        return self.xs[axis].derivative(vhat.transpose(axis, 0), deriv, out_cheby).transpose(axis, 0)


class SpectralSpaceBC(SpectralSpace):
    """Boundary-condition space: the BC basis along ``axis``, plain Chebyshev elsewhere
    (spectralspace.py:69-99)."""

    def __init__(self, bases, axis):
        SpectralSpace.__init__(self, bases)
        self.axis = axis
        for i in range(self.ndim):
            if i == self.axis:
                if hasattr(self.xs[i], "bc"):
                    self.xs[i] = self.xs[i].bc
            elif hasattr(self.xs[i], "family"):
                self.xs[i] = self.xs[i].family
        SpectralSpace.__init__(self, self.xs)
