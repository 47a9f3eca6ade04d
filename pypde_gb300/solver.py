"""Solver plans on the GPU (pypde/solver/{plans,solverplan,matrix,integrator}.py).

Matrices are built on the host at plan time (as in the reference) and turned
into device plans once: banded operators keep only their diagonals, banded LU
factors are swept once, and the fast-diagonalisation Poisson plan factors the
four-diagonal system of every eigenvalue once instead of on every solve.
"""
import ctypes

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._dev import geom, stream, to_dev
from .autodiff import linear, recording
from .bases import MatrixApply
from .host import fdma_lu


def _dense(A):
    if sp.issparse(A):
        A = A.toarray()
    return np.asarray(A)


class Flags:
    def __init__(self, **kwargs):
        self.flags = dict(kwargs)


class MetaPlan:
    """Common plan attributes (plans.py:24-51)."""

    def __init__(self, A, ndim, axis, **kwargs):
        self.A = A
        self.ndim = ndim
        self.axis = axis
        self.N = A.shape[1]
        self._flags = Flags()
        self.flags.update({"axis": axis})

    @property
    def flags(self):
        return self._flags.flags

    def _check_b(self, b):
        assert self.ndim == b.dim(), "Dimensionality mismatch: ndim {:4d} | b.ndim {:4d}. Check ndim.".format(
            self.ndim, b.dim())
        assert self.N == b.shape[self.axis], "Shape mismatch. : N {:4d} | b.shape[axis] {:4d}. Check axis.".format(
            self.N, b.shape[self.axis])


class MatrixBase:
    """Scalar or matrix acting along an axis (matrix.py:7-77)."""

    def __init__(self, M, axis=0, sparse=False):
        self.axis = axis
        self.sparse = sparse
        self.scalar = isinstance(M, (float, int))
        if self.scalar:
            self.value = float(M)
        else:
            self.value = _dense(M)
            self._op = MatrixApply(self.value)

    def dot(self, b):
        b = to_dev(b)
        if self.scalar:
            return self.value * b
        if b.dim() == 1:
            return self._op.apply(b, 0)
        return self._op.apply(b, self.axis)

    @property
    def T(self):
        return self.value if self.scalar else self.value.T


class PlanRHS(MetaPlan):
    """Pre-multiply along an axis (plans.py:54-74)."""

    def __init__(self, A, ndim, axis):
        MetaPlan.__init__(self, A=A, ndim=ndim, axis=axis)
        self.A = MatrixBase(A, axis=self.axis, sparse=True)
        self.flags.update({"method": "multiply"})

    def solve(self, b):
        b = to_dev(b)
        self._check_b(b)
        return self.A.dot(b)


def PlanLHS(A, ndim, axis, method, **kwargs):
    """Plan factory (plans.py:77-119)."""
    methods = {"numpy": Plan_numpy, "twodma": Plan_twodma, "fdma": Plan_fdma, "poisson": Plan_Poisson,
               "multiply": PlanRHS}
    if method not in methods:
        raise ValueError("Method name {:} not found in: {:}".format(method, methods.keys()))
    return methods[method](A=A, ndim=ndim, axis=axis, **kwargs)


class Plan_numpy(MetaPlan):
    """General dense solve (plans.py:122-134): applied as the precomputed inverse."""

    def __init__(self, A, ndim, axis):
        MetaPlan.__init__(self, A=A, ndim=ndim, axis=axis)
        self.flags.update({"method": "numpy"})
        self._inv = MatrixApply(np.linalg.inv(_dense(A)))

    def solve(self, b):
        b = to_dev(b)
        self._check_b(b)
        return self._inv.apply(b, self.axis if b.dim() == 2 else 0)


class _InPlaceBanded(MetaPlan):
    def _sweep(self, b, fn):
        axis = self.axis if b.dim() == 2 else 0
        self._check_b(b)
        p, s0, s1, _, nl = geom(b, axis)
        _lib.check(getattr(_lib.lib(), fn)(self._h, p, s0, s1, nl, axis, stream()), self.flags["method"])
        return b

    def _solve_inplace(self, b):
        """In place, like the Fortran intent(inout).  While autograd records, the solve
        is out of place and its backward is the transposed solve A^T x = g."""
        b = to_dev(b)
        self._check_b(b)
        if recording(b):
            return linear(b, lambda x: self._sweep(x.clone(), "pgx_fdma_solve"),
                          lambda g: self._sweep(g.clone(), "pgx_fdma_solve_t"))
        return self._sweep(b, "pgx_fdma_solve")

    def __del__(self):
        try:
            _lib.lib().pgx_fdma_plan_destroy(self._h)
        except Exception:
            pass


class Plan_twodma(_InPlaceBanded):
    """Upper offset-2 bidiagonal solve (plans.py:137-181), in place."""

    def __init__(self, A, ndim, axis):
        MetaPlan.__init__(self, A=A, ndim=ndim, axis=axis)
        self.flags.update({"method": "twodma"})
        A = _dense(A)
        self.d = np.ascontiguousarray(np.diag(A, 0), dtype=np.float64)
        self.u = np.ascontiguousarray(np.diag(A, 2), dtype=np.float64)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().pgx_twodma_plan_create(self.d.ctypes.data_as(ctypes.c_void_p),
                                                      self.u.ctypes.data_as(ctypes.c_void_p), self.d.size,
                                                      ctypes.byref(h)), "twodma plan")
        self._h = h

    def solve(self, b):
        return self._solve_inplace(b)


class Plan_fdma(_InPlaceBanded):
    """Pre-factored four-diagonal solve (plans.py:184-251), in place."""

    def __init__(self, A, ndim, axis):
        MetaPlan.__init__(self, A=A, ndim=ndim, axis=axis)
        self.flags.update({"method": "fdma"})
        self.l, self.d, self.u1, self.u2 = [np.ascontiguousarray(x) for x in fdma_lu(_dense(A))]
        h = ctypes.c_void_p()
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        _lib.check(_lib.lib().pgx_fdma_plan_create(ptr(self.l), ptr(self.d), ptr(self.u1), ptr(self.u2),
                                                    self.d.size, ctypes.byref(h)), "fdma plan")
        self._h = h

    def solve(self, b):
        return self._solve_inplace(b)


class Plan_Poisson(MetaPlan):
    """(A + alpha_i C) x_i = b_i for every eigenvalue alpha_i (plans.py:254-341).

    The reference factors each four-diagonal system inside every solve
    (fdma.f90:146-195); here all factors are built once and the solve is a
    pure sweep with one CUDA thread per (line, parity) chain.
    """

    def __init__(self, A, alpha, C, ndim, axis, singular=False):
        assert ndim == 2
        MetaPlan.__init__(self, A=A, ndim=ndim, axis=axis)
        self.flags.update({"method": "poisson"})
        self.alpha = np.ascontiguousarray(np.real(alpha), dtype=np.float64)
        self.C = C
        self.singular = singular
        Ah = np.ascontiguousarray(_dense(A), dtype=np.float64)
        Ch = np.ascontiguousarray(_dense(C), dtype=np.float64)
        n = Ah.shape[0]
        h = ctypes.c_void_p()
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        _lib.check(_lib.lib().pgx_poisson_plan_create(ptr(Ah), ptr(Ch), ptr(self.alpha), n, self.alpha.size,
                                                       int(bool(singular)), ctypes.byref(h)), "poisson plan")
        self._h = h
        self.solve = self.solve_fortran

    def solve_fortran(self, b):
        b = to_dev(b)
        if self.alpha.size != b.shape[1 - self.axis]:
            raise ValueError("Size of eigenvalue {:3} array does not match to b {:3}!".format(
                self.alpha.size, b.shape[1 - self.axis]))
        if recording(b):
            return linear(b, lambda x: self._sweep(x.clone(), "pgx_poisson_solve"),
                          lambda g: self._sweep(g.clone(), "pgx_poisson_solve_t"))
        return self._sweep(b, "pgx_poisson_solve")

    def _sweep(self, b, fn):
        if b.dim() != 2 or b.shape[self.axis] != self.N or b.shape[1 - self.axis] != self.alpha.size:
            raise ValueError("poisson: array of shape {} does not match the plan".format(tuple(b.shape)))
        p, s0, s1, _, _ = geom(b, self.axis)
        _lib.check(getattr(_lib.lib(), fn)(self._h, p, s0, s1, self.axis, stream()), "poisson")
        return b

    def __del__(self):
        try:
            _lib.lib().pgx_poisson_plan_destroy(self._h)
        except Exception:
            pass


class SolverPlan:
    """Chains of rhs / old / lhs plans (solverplan.py:4-100)."""

    def __init__(self):
        self.plan_for_lhs = []
        self.plan_for_rhs = []
        self.plan_for_old = []

    def add_rhs(self, plan):
        assert isinstance(plan, PlanRHS)
        self.plan_for_rhs.append(plan)

    def add_old(self, plan):
        assert isinstance(plan, PlanRHS)
        self.plan_for_old.append(plan)

    def add_lhs(self, plan):
        assert isinstance(plan, MetaPlan)
        self.plan_for_lhs.append(plan)

    def solve_rhs(self, b):
        for plan in self.plan_for_rhs:
            b = plan.solve(b)
        return b

    def solve_old(self, b):
        for plan in self.plan_for_old:
            b = plan.solve(b)
        return b

    def solve_lhs(self, b):
        for plan in self.plan_for_lhs:
            b = plan.solve(b)
        return b

    def show_plan(self):
        for title, plans in (("Plans RHS:", self.plan_for_rhs), ("Plans RHS (#2):", self.plan_for_old),
                             ("Plans LHS:", self.plan_for_lhs)):
            if plans:
                print(title)
                for i, p in enumerate(plans):
                    print(i + 1, ")", "Apply method '{:s}' along axis {:1d} ".format(p.flags["method"],
                                                                                    p.flags["axis"]))
                print("")


class Integrator:
    """Time loop (pypde/solver/integrator.py:4-44)."""

    def __init__(self):
        self.time = 0.0

    def update(self):
        raise NotImplementedError

    def callback(self):
        pass

    def iterate(self, maxtime, callback=True, *args, **kwargs):
        eps = 1e-3 * self.dt
        while (self.time + eps) < maxtime:
            self.update(*args, **kwargs)
            self.update_time()
            if self.tsave is not None and (self.time + eps) % self.tsave < self.dt * 0.5:
                self.save()
                if callback:
                    self.callback()

    def update_time(self):
        from .field import Field, MultiField
        if isinstance(self.field, Field):
            self.field.t += self.dt
        elif isinstance(self.field, MultiField):
            self.field.update_time(self.dt)
        else:
            raise ValueError("fields must be of type Field or MultiField.")
        self.time += self.dt

    def save(self):
        self.field.save()
