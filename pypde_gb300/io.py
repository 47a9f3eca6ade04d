"""Checkpoints in pypde's layout (field.py:83-173, rbc2d_base.py:208-228).

pypde writes one HDF5 file per snapshot: per field a group ("temp", "ux", "uy",
"pres" for the Rayleigh-Benard solver) with datasets ``v`` (physical values) and
``vhat`` (coefficients), and at the root ``time``, ``x``, ``y`` and the solver's
``nu``, ``kappa``, ``ra``, ``pr``.  An existing dataset is overwritten in place,
a missing one created (write_single_hdf5, field.py:119-126).

With h5py importable the files are that HDF5 layout.  Without it the same
dataset paths are the keys of a NumPy ``.npz`` archive at the file name with the
suffix ``.npz``: the layout and the values are the same, the container is not
HDF5.
"""
import os

import numpy as np

try:  # optional: the HDF5 container of the reference
    import h5py
except ImportError:  # pragma: no cover - depends on the installation
    h5py = None


def snapshot_name(t, filename=None, leading_str="flow", add_time=True):
    """The reference's default file name: leading_str + "_{t:07.2f}" + ".h5" (field.py:91-96)."""
    if filename is not None:
        return filename
    name = leading_str + ("_{:07.2f}".format(float(t)) if add_time else "")
    return name + ".h5"


def container_path(filename):
    """The file actually written: ``filename`` (HDF5) or ``filename`` with suffix .npz (no h5py)."""
    if h5py is not None:
        return filename
    root, ext = os.path.splitext(filename)
    return (root if ext in (".h5", ".hdf5") else filename) + ".npz"


class Store:
    """Datasets by path ("temp/vhat", "time", ...) in one snapshot file; ``mode`` "a" (create or
    update) or "r"."""

    def __init__(self, filename, mode="a"):
        self.path, self.mode = container_path(filename), mode
        if h5py is not None:
            self.hf = h5py.File(self.path, mode)
            self.data = None
        else:
            self.hf = None
            if os.path.exists(self.path):
                with np.load(self.path) as z:
                    self.data = {k: z[k] for k in z.files}
            elif mode == "r":
                raise FileNotFoundError(self.path)
            else:
                self.data = {}

    def __contains__(self, name):
        return name in self.hf if self.hf is not None else name in self.data

    def write(self, name, value):
        value = np.asarray(value)
        if self.hf is not None:
            if name not in self.hf:
                self.hf.create_dataset(name, data=value)
            else:
                self.hf[name][...] = value
        else:
            self.data[name] = value

    def read(self, name):
        if name not in self:
            raise KeyError("%s has no dataset %s" % (self.path, name))
        return np.array(self.hf[name]) if self.hf is not None else np.array(self.data[name])

    def close(self):
        if self.hf is not None:
            self.hf.close()
        elif self.mode != "r":
            np.savez(self.path, **self.data)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _host(x):
    return x.detach().cpu().numpy() if hasattr(x, "detach") else np.asarray(x)


def write_field(field, store, grp_name="", extra=None):
    """Field.write (field.py:83-117) into an open Store."""
    g = grp_name + "/" if grp_name and not grp_name.endswith("/") else grp_name
    store.write(g + "v", _host(field.v))
    store.write(g + "vhat", _host(field.vhat))
    store.write("time", float(field.t))
    store.write("x", np.asarray(field.x))
    if field.ndim > 1:
        store.write("y", np.asarray(field.y))
    for key, val in (extra or {}).items():
        store.write(key, val)


def read_field(field, store, grp_name="", extra=None):
    """Field.read (field.py:137-173) from an open Store; ``extra`` keys are filled in place."""
    g = grp_name + "/" if grp_name and not grp_name.endswith("/") else grp_name
    field.v = store.read(g + "v")
    field.vhat = store.read(g + "vhat")
    field.t = float(store.read("time"))
    for key in list((extra or {}).keys()):
        extra[key] = store.read(key)
