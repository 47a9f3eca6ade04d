"""Import shims that let the unmodified pypde reference run in this container.

Used only by ``make_golden.py`` (and the reference-pinning CPU test) to run
the reference itself and record golden vectors.  Nothing here is used by the GPU
tests, the benchmark or the product package.

* The four f2py Fortran modules (differentiate_cheby, tdma, fdma, twodma) are
  restated statement-by-statement from their ``.f90`` sources, with f2py's
  calling conventions: ``intent(inout)`` arrays are updated in place and must
  be Fortran-contiguous float64, ``intent(out)`` arrays are returned freshly
  zero-filled, ``intent(in)`` reals are cast to float64.  The shipped
  compiled ``.so`` files are never loaded.
* matplotlib / h5py / pypde.plot are stubbed (plotting and HDF5 I/O are not
  on the time-step path).
* ``numpy.linalg.eig`` is wrapped to return real arrays when every imaginary
  part is exactly zero, which is what NumPy 1.x (the reference's environment)
  did and what its f2py calls rely on: the Poisson plan feeds eig's output to
  a ``real(8), intent(inout)`` Fortran argument (plans.py:310-314).
"""
import os
import sys
import types
import warnings

import numpy as np

# Where the pypde checkout lives: the PYPDE_REFERENCE environment variable, or the
# --reference argument of the generating scripts.
REFERENCE = os.environ.get("PYPDE_REFERENCE")


def _f_inout(x, name):
    if not isinstance(x, np.ndarray) or x.dtype != np.float64:
        raise ValueError("failed to initialize intent(inout) array %s: not float64" % name)
    if x.ndim > 1 and not x.flags.f_contiguous:
        raise ValueError("failed to initialize intent(inout) array %s: not fortran contiguous" % name)


def _real(a):
    a = np.asarray(a)
    if np.iscomplexobj(a):
        warnings.warn("Casting complex values to real discards the imaginary part",
                      np.exceptions.ComplexWarning)
        a = a.real
    return np.asarray(a, dtype=np.float64)


# ---------------------------------------------------------------- differentiate_cheby.f90
def diff_1d(c):
    c = _real(c)
    n = c.shape[0]
    dc = np.zeros(n)
    # Fortran: dc(n-1) = 2*(n-1)*c(n); do i=n-2,2,-1: dc(i) = dc(i+2) + 2*i*c(i+1); dc(1) = dc(3)/2. + c(2)
    dc[n - 2] = 2 * (n - 1) * c[n - 1]
    for i in range(n - 2, 1, -1):
        dc[i - 1] = dc[i + 1] + 2 * i * c[i]
    dc[0] = dc[2] / 2.0 + c[1]
    return dc


def diff_2d(c):
    c = _real(c)
    n, m = c.shape
    dc = np.zeros((n, m), order="F")
    dc[n - 2, :] = 2 * (n - 1) * c[n - 1, :]
    for i in range(n - 2, 1, -1):
        dc[i - 1, :] = dc[i + 1, :] + 2 * i * c[i, :]
    dc[0, :] = dc[2, :] / 2.0 + c[1, :]
    return dc


# ---------------------------------------------------------------- tdma.f90
def _tdma(a, b, c, d, k):
    n = b.shape[0]
    w = np.zeros(n - k)
    g = np.zeros(d.shape)
    for i in range(1, n - k + 1):  # Fortran i = 1..n-k
        if i < k + 1:
            w[i - 1] = c[i - 1] / b[i - 1]
        else:
            w[i - 1] = c[i - 1] / (b[i - 1] - a[i - k - 1] * w[i - k - 1])
    for i in range(1, n + 1):
        if i < k + 1:
            g[i - 1] = d[i - 1] / b[i - 1]
        else:
            g[i - 1] = (d[i - 1] - a[i - k - 1] * g[i - k - 1]) / (b[i - 1] - a[i - k - 1] * w[i - k - 1])
    x = np.zeros(d.shape, order="F")
    x[n - k - 1:n] = g[n - k - 1:n]  # x(n-k:n) = g(n-k:n)
    for i in range(n - k + 1, 1, -1):  # do i=n-k+1,2,-1
        x[i - 2] = g[i - 2] - w[i - 2] * x[i + k - 2]
    return x


def solve_tdma_1d(a, b, c, d, k):
    return _tdma(_real(a), _real(b), _real(c), _real(d), int(k))


def solve_tdma_2d(a, b, c, d, k):
    return _tdma(_real(a), _real(b), _real(c), _real(d), int(k))


# ---------------------------------------------------------------- twodma.f90
def _twodma_axis0(d, u, x):
    n = x.shape[0]
    x[n - 1] = x[n - 1] / d[n - 1]
    x[n - 2] = x[n - 2] / d[n - 2]
    for i in range(n - 2, 0, -1):  # do i=n-2,1,-1
        x[i - 1] = (x[i - 1] - u[i - 1] * x[i + 1]) / d[i - 1]


def solve_twodma_1d(d, u, x):
    _f_inout(x, "x")
    _twodma_axis0(_real(d), _real(u), x)


def solve_twodma_2d(d, u1, x, axis):
    _f_inout(x, "x")
    if axis == 0:
        _twodma_axis0(_real(d), _real(u1), x)
    elif axis == 1:
        _twodma_axis0(_real(d), _real(u1), x.T)


# ---------------------------------------------------------------- fdma.f90
def _fdma_axis0(l, d, u1, u2, x):
    n = x.shape[0]
    for i in range(3, n + 1):  # do i=3,n
        x[i - 1] = x[i - 1] - l[i - 3] * x[i - 3]
    x[n - 1] = x[n - 1] / d[n - 1]
    x[n - 2] = x[n - 2] / d[n - 2]
    x[n - 3] = (x[n - 3] - u1[n - 3] * x[n - 1]) / d[n - 3]
    x[n - 4] = (x[n - 4] - u1[n - 4] * x[n - 2]) / d[n - 4]
    for i in range(n - 4, 0, -1):  # do i=n-4,1,-1
        x[i - 1] = (x[i - 1] - u1[i - 1] * x[i + 1] - u2[i - 1] * x[i + 3]) / d[i - 1]


def solve_fdma_1d(l, d, u1, u2, x):
    _f_inout(x, "x")
    _fdma_axis0(_real(l), _real(d), _real(u1), _real(u2), x)


def solve_fdma_2d(l, d, u1, u2, x, axis):
    _f_inout(x, "x")
    if axis == 0:
        _fdma_axis0(_real(l), _real(d), _real(u1), _real(u2), x)
    elif axis == 1:
        _fdma_axis0(_real(l), _real(d), _real(u1), _real(u2), x.T)


def init_fdma(A):
    A = _real(A)
    n = A.shape[0]
    d, u1, u2, l = np.zeros(n), np.zeros(n - 2), np.zeros(n - 4), np.zeros(n - 2)
    for i in range(1, n + 1):
        d[i - 1] = A[i - 1, i - 1]
        if i > 2:
            l[i - 3] = A[i - 1, i - 3]
        if i < n - 1:
            u1[i - 1] = A[i - 1, i + 1]
        if i < n - 3:
            u2[i - 1] = A[i - 1, i + 3]
    for i in range(3, n + 1):
        l[i - 3] = l[i - 3] / d[i - 3]
        d[i - 1] = d[i - 1] - l[i - 3] * u1[i - 3]
        if i < n - 1:
            u1[i - 1] = u1[i - 1] - l[i - 3] * u2[i - 3]
    return d, u1, u2, l


def solve_fdma_type2(A, C, lam, x, axis, singular):
    _f_inout(x, "x")
    A, C, lam = _real(A), _real(C), _real(lam)
    n, m = x.shape
    if axis == 0:
        for i in range(m):
            if singular and abs(lam[i]) < 1e-10:
                d, u1, u2, l = init_fdma(A[1:, 1:] + C[1:, 1:] * lam[i])
                col = x[1:, i]
                _fdma_axis0(l, d, u1, u2, col)
                x[0, i] = 0.0
            else:
                d, u1, u2, l = init_fdma(A + C * lam[i])
                col = x[:, i]
                _fdma_axis0(l, d, u1, u2, col)
    elif axis == 1:
        for i in range(n):
            d, u1, u2, l = init_fdma(A + C * lam[i])
            row = x[i, :]
            _fdma_axis0(l, d, u1, u2, row)


# ---------------------------------------------------------------- installation
def _module(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    return m


def install(reference=REFERENCE):
    """Register the shims and stubs, patch eig, and put the reference on sys.path."""
    if not reference or not os.path.isdir(os.path.join(reference, "pypde")):
        raise SystemExit("pypde reference checkout not found: pass --reference PATH or set PYPDE_REFERENCE "
                         "(got %r)" % (reference,))
    anything = lambda *a, **k: None  # noqa: E731
    stub = _module("stub")
    for name in ["matplotlib", "matplotlib.pyplot", "matplotlib.animation", "mpl_toolkits",
                 "mpl_toolkits.mplot3d", "h5py"]:
        m = _module(name)
        m.__getattr__ = lambda attr: anything
        sys.modules[name] = m
    plot = _module("pypde.plot", initplot=anything, plot=anything)
    plot.__path__ = []
    sys.modules["pypde.plot"] = plot
    sys.modules["pypde.plot.initplot"] = _module("pypde.plot.initplot", initplot=anything)
    sys.modules["pypde.plot.wireframe"] = _module("pypde.plot.wireframe", plot=anything)
    sys.modules["pypde.plot.anim"] = _module("pypde.plot.anim", animate_line=anything,
                                             animate_contour=anything, animate_wireframe=anything)
    del stub
    for pkg in ["pypde.bases.fortran", "pypde.bases.linalg.fortran", "pypde.solver.linalg.fortran"]:
        m = _module(pkg)
        m.__path__ = []
        sys.modules[pkg] = m
    sys.modules["pypde.bases.fortran.differentiate_cheby"] = _module(
        "differentiate_cheby", diff_1d=diff_1d, diff_2d=diff_2d)
    sys.modules["pypde.bases.linalg.fortran.tdma"] = _module(
        "tdma", solve_tdma_1d=solve_tdma_1d, solve_tdma_2d=solve_tdma_2d)
    sys.modules["pypde.solver.linalg.fortran.twodma"] = _module(
        "twodma", solve_twodma_1d=solve_twodma_1d, solve_twodma_2d=solve_twodma_2d)
    sys.modules["pypde.solver.linalg.fortran.fdma"] = _module(
        "fdma", solve_fdma_1d=solve_fdma_1d, solve_fdma_2d=solve_fdma_2d,
        init_fdma=init_fdma, solve_fdma_type2=solve_fdma_type2)
    for pkg, sub in [("pypde.bases.fortran", "differentiate_cheby"),
                     ("pypde.bases.linalg.fortran", "tdma"),
                     ("pypde.solver.linalg.fortran", "twodma"),
                     ("pypde.solver.linalg.fortran", "fdma")]:
        setattr(sys.modules[pkg], sub, sys.modules[pkg + "." + sub])

    if not getattr(np.linalg.eig, "_numpy1_semantics", False):
        _eig = np.linalg.eig

        def eig(a):
            w, v = _eig(a)
            if np.iscomplexobj(w) and np.all(w.imag == 0.0):
                w, v = w.real.copy(), v.real.copy()
            return w, v

        eig._numpy1_semantics = True
        np.linalg.eig = eig

    for p in (reference, reference + "/navier"):
        if p not in sys.path:
            sys.path.insert(0, p)
    warnings.simplefilter("ignore", np.exceptions.ComplexWarning)
