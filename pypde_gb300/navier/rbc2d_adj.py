"""Adjoint-descent steady-state search on the GPU (navier/rbc2d_adj.py).

Each ``update()``: one forward NavierStokes step gives the residual
F = (Phi(X) - X) / dt; three Poisson solves smooth it (nabla^-2 F / nu, / kappa);
X then moves along the adjoint-linearised convection, the buoyancy transpose
and F, followed by a pressure projection.  Built from the same device
operations as the plain path.
"""
import numpy as np

from ..bases import Base
from ..field import Field
from ..field_operations import cheby_to_galerkin, conv_term, convective_term, galerkin_to_cheby
from ..solver import Integrator
from ..templates import solverplan_poisson2d
from .rbc2d import NavierStokes, NavierStokesBase


class NavierStokesAdjoint(NavierStokesBase, Integrator):
    """NavierStokesAdjoint (rbc2d_adj.py:15-356), IMEX Euler coefficients."""

    avail_cases = ["rbc", "linear", "zero"]

    def __init__(self, case="rbc", **kwargs):
        if case not in self.avail_cases:
            raise ValueError("Specified case is not available: ", self.avail_cases)
        self.case = case
        Integrator.__init__(self)
        NavierStokesBase.__init__(self, **kwargs)
        self.NS = NavierStokes(case=case, **self.CONFIG)
        if self.NS.nstage != 1:
            raise NotImplementedError("the adjoint-descent step is provided for the Euler coefficients")
        side = "CN" if case == "rbc" else "CD"
        N, M = self.shape
        mk = lambda kx: Field([Base(N, kx, dealias=3 / 2), Base(M, "CD", dealias=3 / 2)])  # noqa: E731
        self.T, self.U, self.V = mk(side), mk("CD"), mk("CD")
        self.TA, self.UA, self.VA = mk(side), mk("CD"), mk("CD")
        self.P = Field([Base(N, "CN"), Base(M, "CN")])
        self.pres = Field([Base(N, "CH"), Base(M, "CH")])
        self.setup_solver()
        self.Tbc = self.NS.Tbc
        tb = galerkin_to_cheby(self.NS.Tbc.vhat, self.NS.Tbc)
        self.temp_bc = self.deriv_field.dealias.backward(tb) if self.dealias else self.deriv_field.backward(tb)

    def setup_solver(self):
        """Stage coefficients and pressure plan of the forward solver; smoothing plans (rbc2d_adj.py:129-144)."""
        self.a, self.b, self.c, self.nstage = self.NS.a, self.NS.b, self.NS.c, self.NS.nstage
        self.solver_P = self.NS.solver_P
        self.nabla_U = solverplan_poisson2d(self.U.xs, singular=False, scale=self.scale)
        self.nabla_V = solverplan_poisson2d(self.V.xs, singular=False, scale=self.scale)
        self.nabla_T = solverplan_poisson2d(self.T.xs, singular=False, scale=self.scale)

    def _phys(self, F):
        return F.dealias.backward(F.vhat) if self.dealias else F.backward(F.vhat)

    def conv(self, field, u, deriv):
        return conv_term(field, u, deriv=deriv, deriv_field=self.deriv_field, dealias=self.dealias,
                         scale=self.scale)

    def _forward(self, conv):
        return self.deriv_field.dealias.forward(conv) if self.dealias else self.deriv_field.forward(conv)

    def conv_term_adj(self, deriv, ux, uz, temp):
        """Adjoint convection, x or z component (rbc2d_adj.py:162-187)."""
        c = self.conv(self.UA, ux, deriv)
        c = c + self.conv(self.VA, uz, deriv)
        c = c + self.conv(self.TA, temp, deriv)
        c = c + self.conv(self.TA, self.temp_bc, deriv)
        return self._forward(c)

    def update_NS(self):
        """Residual F of one forward step, then its inverse-Laplacian smoothing (rbc2d_adj.py:189-205)."""
        ns = self.NS
        ns.U.vhat, ns.V.vhat, ns.T.vhat = self.U.vhat.clone(), self.V.vhat.clone(), self.T.vhat.clone()
        ns.update()
        ns.U.vhat = (ns.U.vhat - self.U.vhat) / self.dt
        ns.V.vhat = (ns.V.vhat - self.V.vhat) / self.dt
        ns.T.vhat = (ns.T.vhat - self.T.vhat) / self.dt
        for plan, F, FA, coef in ((self.nabla_U, ns.U, self.UA, self.nu), (self.nabla_V, ns.V, self.VA, self.nu),
                                  (self.nabla_T, ns.T, self.TA, self.kappa)):
            FA.vhat = plan.solve_lhs(plan.solve_rhs(galerkin_to_cheby(F.vhat, F))) / coef

    def _conv_ns(self, FA, ux, uz):
        return convective_term(FA, ux, uz, deriv_field=self.deriv_field, dealias=self.dealias, scale=self.scale)

    def update(self):
        """One adjoint-descent step (rbc2d_adj.py:321-356)."""
        ns = self.NS
        for rk in range(self.nstage):
            a, b = self.a[rk], self.b[rk]
            ux, uz, temp = self._phys(self.U), self._phys(self.V), self._phys(self.T)
            self.update_NS()
            for F, d, FA, FN in ((self.U, (1, 0), self.UA, ns.U), (self.V, (0, 1), self.VA, ns.V)):
                rhs = -a * self.grad(self.pres, deriv=d)
                rhs = rhs + b * self._conv_ns(FA, ux, uz)
                rhs = rhs + b * self.conv_term_adj(d, ux, uz, temp)
                rhs = rhs + a * galerkin_to_cheby(FN.vhat, F)
                F.vhat = F.vhat + self.dt * cheby_to_galerkin(rhs, F)
            div = ns.divergence_velocity(self.U, self.V)
            self.P.vhat = self.solver_P.solve_lhs(self.solver_P.solve_rhs(div))
            self.P.vhat[0, 0] = 0
            self.pres.vhat = self.pres.vhat + galerkin_to_cheby(self.P.vhat, self.P) / (self.dt * a)
            self.U.vhat = self.U.vhat - cheby_to_galerkin(self.grad(self.P, deriv=(1, 0)), self.U)
            self.V.vhat = self.V.vhat - cheby_to_galerkin(self.grad(self.P, deriv=(0, 1)), self.V)
            rhs = b * self._conv_ns(self.TA, ux, uz)
            rhs = rhs + a * galerkin_to_cheby(ns.T.vhat, self.T)
            rhs = rhs + a * galerkin_to_cheby(self.VA.vhat, self.VA)
            self.T.vhat = self.T.vhat + self.dt * cheby_to_galerkin(rhs, self.T)

    def residual_norms(self):
        """|F_U|, |F_V|, |F_T| of the last update (rbc2d_adj.py:316-319)."""
        return tuple(float(np.linalg.norm(f.vhat.detach().cpu().numpy())) for f in (self.NS.U, self.NS.V, self.NS.T))
