"""Adjoint-descent steady-state step restated in NumPy (oracle, test infrastructure).

Reference: navier/rbc2d_adj.py (NavierStokesAdjoint).  One update runs a
forward NavierStokes step to get the residual F = (Phi(X) - X)/dt, smooths it
with an inverse Laplacian (three Poisson solves, divided by nu or kappa),
and moves X along the adjoint-linearised convection + buoyancy transpose +
F, with a pressure projection.
"""
import numpy as np

from . import field as fo
from . import rbc2d as orb
from . import solver as so


class NavierStokesAdjoint:
    """NavierStokesAdjoint (rbc2d_adj.py:15-356)."""

    def __init__(self, case="rbc", **kwargs):
        self.NS = orb.NavierStokes(case=case, **kwargs)
        ns = self.NS
        self.case = case
        for k in ("shape", "dt", "nu", "kappa", "scale", "dealias", "a", "b", "c", "nstage"):
            setattr(self, k, getattr(ns, k))
        N, M = self.shape
        self.Tsp, self.Usp, self.Psp, self.deriv = ns.Tsp, ns.Usp, ns.Psp, ns.deriv
        self.That = np.zeros(self.Tsp.M)
        self.Uhat = np.zeros(self.Usp.M)
        self.Vhat = np.zeros(self.Usp.M)
        self.Phat = np.zeros(self.Psp.M)
        self.pres = np.zeros((N, M))
        # setup_solver (rbc2d_adj.py:129-144): smoothing Poisson plans, singular=False
        self.nabla_U = so.Poisson2D(self.Usp.keys, (N, M), singular=False, scale=self.scale)
        self.nabla_T = so.Poisson2D(self.Tsp.keys, (N, M), singular=False, scale=self.scale)
        # temperature BC on the (dealiased) physical grid (rbc2d_adj.py:104-116)
        tb = fo.galerkin_to_cheby(ns.Tbcsp, ns.Tbc_vhat)
        self.temp_bc = self.deriv.dealias_backward(tb) if self.dealias else self.deriv.backward(tb)

    def _phys(self, space, vhat):
        return space.dealias_backward(vhat) if self.dealias else space.backward(vhat)

    def conv(self, space, vhat, u, deriv):
        return fo.conv_term(space, vhat, u, deriv, self.deriv, self.dealias, self.scale)

    def _fwd(self, conv):
        return self.deriv.dealias_forward(conv) if self.dealias else self.deriv.forward(conv)

    def conv_term_adj(self, deriv, ux, uz, temp):
        """conv_term_adj_ux / _uz (rbc2d_adj.py:162-187)."""
        c = self.conv(self.Usp, self.UA, ux, deriv)
        c = c + self.conv(self.Usp, self.VA, uz, deriv)
        c = c + self.conv(self.Tsp, self.TA, temp, deriv)
        c = c + self.conv(self.Tsp, self.TA, self.temp_bc, deriv)
        return self._fwd(c)

    def update_NS(self):
        """Residual of one forward step and its H^-1 smoothing (rbc2d_adj.py:189-205)."""
        ns = self.NS
        ns.Uhat, ns.Vhat, ns.That = self.Uhat.copy(), self.Vhat.copy(), self.That.copy()
        ns.update()
        self.FU = (ns.Uhat - self.Uhat) / self.dt
        self.FV = (ns.Vhat - self.Vhat) / self.dt
        self.FT = (ns.That - self.That) / self.dt
        smooth = lambda plan, sp, F: plan.solve_lhs(plan.solve_rhs(fo.galerkin_to_cheby(sp, F)))  # noqa: E731
        self.UA = smooth(self.nabla_U, self.Usp, self.FU) / self.nu
        self.VA = smooth(self.nabla_U, self.Usp, self.FV) / self.nu
        self.TA = smooth(self.nabla_T, self.Tsp, self.FT) / self.kappa

    def update(self):
        """One adjoint-descent step (rbc2d_adj.py:321-356)."""
        ns = self.NS
        for rk in range(self.nstage):
            a, b = self.a[rk], self.b[rk]
            ux = self._phys(self.Usp, self.Uhat)
            uz = self._phys(self.Usp, self.Vhat)
            temp = self._phys(self.Tsp, self.That)
            self.update_NS()
            g = lambda sp, v, d: fo.grad(sp, v, d, self.scale)  # noqa: E731
            # update_U / update_V (rbc2d_adj.py:207-259)
            rhs = -a * g(self.deriv, self.pres, (1, 0))
            rhs = rhs + b * fo.convective_term(self.Usp, self.UA, ux, uz, self.deriv, dealias=self.dealias,
                                               scale=self.scale)
            rhs = rhs + b * self.conv_term_adj((1, 0), ux, uz, temp)
            rhs = rhs + a * fo.galerkin_to_cheby(self.Usp, self.FU)
            self.Uhat = self.Uhat + self.dt * fo.cheby_to_galerkin(self.Usp, rhs)
            rhs = -a * g(self.deriv, self.pres, (0, 1))
            rhs = rhs + b * fo.convective_term(self.Usp, self.VA, ux, uz, self.deriv, dealias=self.dealias,
                                               scale=self.scale)
            rhs = rhs + b * self.conv_term_adj((0, 1), ux, uz, temp)
            rhs = rhs + a * fo.galerkin_to_cheby(self.Usp, self.FV)
            self.Vhat = self.Vhat + self.dt * fo.cheby_to_galerkin(self.Usp, rhs)
            # pressure projection (rbc2d_adj.py:283-300)
            div = g(self.Usp, self.Uhat, (1, 0)) + g(self.Usp, self.Vhat, (0, 1))
            self.Phat = ns.solver_P.solve_lhs(ns.solver_P.solve_rhs(div))
            self.Phat[0, 0] = 0
            self.pres = self.pres + fo.galerkin_to_cheby(self.Psp, self.Phat) / (self.dt * a)
            self.Uhat = self.Uhat - fo.cheby_to_galerkin(self.Usp, g(self.Psp, self.Phat, (1, 0)))
            self.Vhat = self.Vhat - fo.cheby_to_galerkin(self.Usp, g(self.Psp, self.Phat, (0, 1)))
            # update_T (rbc2d_adj.py:261-281)
            rhs = b * fo.convective_term(self.Tsp, self.TA, ux, uz, self.deriv, dealias=self.dealias,
                                         scale=self.scale)
            rhs = rhs + a * fo.galerkin_to_cheby(self.Tsp, self.FT)
            rhs = rhs + a * fo.galerkin_to_cheby(self.Usp, self.VA)
            self.That = self.That + self.dt * fo.cheby_to_galerkin(self.Tsp, rhs)
