"""Rayleigh-Benard IMEX time stepper on the GPU (navier/rbc2d.py, navier/rbc2d_base.py).

``NavierStokes.update()`` takes one time step.  Unless autograd records
through the state it runs the fused form (``NavierStokes.fused()``): the same
step as about a dozen fused line-program passes that can be replayed from a
CUDA graph (``pypde_gb300.navier.fused``).  ``update(fused=False)`` follows the
reference operation by operation, every pypde call (grad, convective_term,
solver plans) one or a few launches of the pgx kernels: the *plain* path, which
``torch.autograd`` differentiates.
"""
import numpy as np
import torch

from .._dev import to_host
from ..bases import Base
from ..field import Field, FieldBC, MultiField
from ..field_operations import avg_vol, avg_x, cheby_to_galerkin, convective_term, galerkin_to_cheby, grad
from ..solver import Integrator
from ..templates import solverplan_hholtz2d_adi, solverplan_poisson2d
from .steady import NavierStokesSteadyState

CONFIG = {"shape": (50, 50), "ra": 5e3, "pr": 1.0, "dt": 0.2, "ndim": 2, "tsave": 0.1, "dealias": True,
          "integrator": "eu", "beta": 1.0, "aspect": 1.0}


def nu(Ra, Pr, L):
    return np.sqrt(Pr / (Ra / L ** 3.0))


def kappa(Ra, Pr, L):
    return np.sqrt(1 / Pr / (Ra / L ** 3.0))


def transfer_function(TL, TM, TR, x, k=0.01):
    """Smooth sidewall temperature profile (rbc2d.py:437-446)."""
    x = np.asarray(x)
    xs = x * 2.0 / (x[-1] - x[0])
    left = -k * xs / (k + xs + 1) * (TL - TM) + TM
    right = k * xs / (k - xs + 1) * (TR - TM) + TM
    return np.where(xs < 0, left, right)


class NavierStokesBase:
    """Configuration, nu / kappa, time-step coefficients (rbc2d_base.py:24-114)."""

    def __init__(self, **kwargs):
        if "Ra" in kwargs or "Pr" in kwargs:
            raise ValueError("Use small ra/pr!")
        self.CONFIG = dict(CONFIG)
        self.CONFIG.update(**kwargs)
        self.__dict__.update(**self.CONFIG)
        self.normalize = True
        self.set_nu_kappa()
        self.deriv_field = Field([Base(self.shape[0], "CH", dealias=3 / 2), Base(self.shape[1], "CH", dealias=3 / 2)])
        self.x = self.deriv_field.x * self.scale[0]
        self.y = self.deriv_field.y * self.scale[1]
        self.xx, self.yy = np.meshgrid(self.x, self.y, indexing="ij")

    def set_nu_kappa(self, normalize=None):
        if normalize is None:
            normalize = self.normalize
        L = 1.0 if normalize else 2.0
        self.nu = nu(self.ra, self.pr, L=L)
        self.kappa = kappa(self.ra, self.pr, L=L)
        self.scale = (self.aspect * 0.5, 0.5) if normalize else (self.aspect * 1.0, 1.0)

    def grad(self, field, deriv, return_field=False):
        return grad(field, deriv=deriv, return_field=return_field, scale=self.scale)

    def set_timestep_coefficients_rk3(self):
        self.nstage = 3
        self.a = np.array([8.0 / 15.0, 2.0 / 15.0, 1.0 / 3.0])
        self.b = np.array([8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0])
        self.c = np.array([0, -17.0 / 60.0, -5.0 / 12.0])

    def set_timestep_coefficients_euler(self):
        self.nstage = 1
        self.a = np.array([1.0])
        self.b = np.array([1.0])
        self.c = np.array([0])

    # -- diagnostics (rbc2d_base.py:344-386)
    def eval_Nu(self):
        Lz = self.y[-1] - self.y[0]
        return eval_Nu(self.T, self.deriv_field, Tbc=self.Tbc, Lz=Lz), eval_Nuvol(
            self.T, self.V, self.kappa, self.deriv_field, Tbc=self.Tbc, Lz=Lz)

    def eval_KE(self):
        """0.5 avg_vol(u^2 + v^2) on the physical grid (pypde defines no kinetic energy)."""
        u = self.U.backward(self.U.vhat)
        v = self.V.backward(self.V.vhat)
        return float(0.5 * avg_vol(u * u + v * v, self.deriv_field.dx, self.deriv_field.dy))


def _dT(T, field, Lz, Tbc):
    Tv = T.backward(T.vhat)
    if Tbc is not None:
        Tv = Tv + Tbc.v
    That = field.forward(Tv)
    dThat = field.derivative(That, 1, axis=1) / (Lz / 2.0)
    return Tv, field.backward(dThat)


def eval_Nu(T, field, Lz=1.0, Tbc=None):
    """Mean of bottom and top plate Nusselt numbers (rbc2d_base.py:344-363)."""
    _, dT = _dT(T, field, Lz, Tbc)
    dTavg = avg_x(dT, field.dx)
    return float((-dTavg[0] * Lz - dTavg[-1] * Lz) / 2.0)


def eval_Nuvol(T, V, kappa, field, Lz=1.0, Tbc=None):
    """Volume-averaged heat flux (rbc2d_base.py:366-386)."""
    Tv, dT = _dT(T, field, Lz, Tbc)
    Vv = V.backward(V.vhat)
    return float(avg_vol((Tv * Vv / kappa - dT) * Lz, field.dx, field.dy))


class NavierStokes(NavierStokesBase, NavierStokesSteadyState, Integrator):
    """Boussinesq convection, IMEX Euler / RK3 with pressure projection (rbc2d.py:28-434)."""

    avail_cases = ["rbc", "linear", "zero"]

    def __init__(self, case="rbc", **kwargs):
        if case not in self.avail_cases:
            raise ValueError("Specified case is not available: ", self.avail_cases)
        self.case = case
        NavierStokesBase.__init__(self, **kwargs)
        Integrator.__init__(self)
        side = "CN" if case == "rbc" else "CD"
        self.set_fieldbc = self.set_temp_fieldbc_zero if case == "zero" else self.set_temp_fieldbc_linear
        N, M = self.shape
        self.T = Field([Base(N, side, dealias=3 / 2), Base(M, "CD", dealias=3 / 2)])
        self.U = Field([Base(N, "CD", dealias=3 / 2), Base(M, "CD", dealias=3 / 2)])
        self.V = Field([Base(N, "CD", dealias=3 / 2), Base(M, "CD", dealias=3 / 2)])
        self.P = Field([Base(N, "CN"), Base(M, "CN")])
        self.pres = Field([Base(N, "CH"), Base(M, "CH")])
        self.field = MultiField([self.T, self.U, self.V, self.pres], ["temp", "ux", "uy", "pres"])
        self.setup_solver()
        self.set_fieldbc()
        self._fused = None

    def reset(self, reset_time=True):
        self.set_nu_kappa()
        self.setup_solver()
        self._fused = None
        if reset_time:
            self.reset_time()

    def reset_time(self):
        self.time = 0.0
        for f in self.field.fields:
            f.t = 0.0

    def set_temp_fieldbc_linear(self):
        bc = np.zeros((self.shape[0], 2))
        bc[:, 0], bc[:, 1] = 0.5, -0.5
        self._set_fieldbc(bc, axis=1)

    def set_temp_fieldbc_zero(self):
        bc = np.zeros((2, self.shape[1]))
        bc[0, :] = transfer_function(0.5, 0, -0.5, self.y, k=0.02)
        bc[1, :] = bc[0, :]
        self._set_fieldbc(bc, axis=0)

    def _set_fieldbc(self, bc, axis):
        """Inhomogeneous temperature lift and its derivatives (rbc2d.py:135-178)."""
        self.Tbc = FieldBC(self.T.xs, axis=axis)
        self.Tbc.add_bc(bc)
        self.dTbcdz2 = self.grad(self.Tbc, deriv=(0, 2))
        vhat = self.grad(self.Tbc, deriv=(0, 1))
        self.dTbcdz1 = self.deriv_field.dealias.backward(vhat) if self.dealias else self.deriv_field.backward(vhat)
        self.Tbc_cheby = galerkin_to_cheby(self.Tbc.vhat, self.Tbc)

    def setup_solver(self):
        """Helmholtz plans per stage and the Poisson plan (rbc2d.py:180-211)."""
        if self.integrator == "rk3":
            self.set_timestep_coefficients_rk3()
        else:
            self.set_timestep_coefficients_euler()
        self.solver_U, self.solver_V, self.solver_T = [], [], []
        for rk in range(self.nstage):
            lu = self.dt * self.a[rk] * self.beta * self.nu
            lt = self.dt * self.a[rk] * self.beta * self.kappa
            self.solver_U.append(solverplan_hholtz2d_adi(bases=self.U.xs, lam=lu, scale=self.scale))
            self.solver_V.append(solverplan_hholtz2d_adi(bases=self.V.xs, lam=lu, scale=self.scale))
            self.solver_T.append(solverplan_hholtz2d_adi(bases=self.T.xs, lam=lt, scale=self.scale))
        self.solver_P = solverplan_poisson2d(self.P.xs, singular=True, scale=self.scale)

    # ------------------------------------------------------------ plain step
    def update_velocity(self, p, u, v, fac=1.0):
        dpdx = self.grad(p, deriv=(1, 0))
        dpdz = self.grad(p, deriv=(0, 1))
        u.vhat = u.vhat - cheby_to_galerkin(dpdx * fac, u)
        v.vhat = v.vhat - cheby_to_galerkin(dpdz * fac, v)

    def divergence_velocity(self, u, v):
        return self.grad(u, deriv=(1, 0)) + self.grad(v, deriv=(0, 1))

    def conv_term(self, field, ux, uz, add_bc=None):
        return convective_term(field, ux, uz, deriv_field=self.deriv_field, add_bc=add_bc, dealias=self.dealias,
                               scale=self.scale)

    def _explicit_diffusion(self, F, coef, stage):
        f = self.dt * self.a[stage] * (1 - self.beta) * coef
        return f * self.grad(F, deriv=(2, 0)) + f * self.grad(F, deriv=(0, 2))

    def _helmholtz(self, solver, rhs, F):
        rhs = solver.solve_rhs(rhs)
        rhs = rhs + solver.solve_old(F.vhat)
        F.vhat = solver.solve_lhs(rhs)

    def update_U(self, stage):
        rhs = -self.dt * self.a[stage] * self.grad(self.pres, deriv=(1, 0))
        rhs = rhs - self.dt * self.b[stage] * self.conv_term(self.U, self.ux, self.uz)
        if self.c[stage] != 0:
            rhs = rhs - self.dt * self.c[stage] * self.conv_term(self.U, self.ux_old, self.uz_old)
        if self.beta != 1.0:
            rhs = rhs + self._explicit_diffusion(self.U, self.nu, stage)
        self._helmholtz(self.solver_U[stage], rhs, self.U)

    def update_V(self, That, stage):
        rhs = -self.dt * self.a[stage] * self.grad(self.pres, deriv=(0, 1))
        rhs = rhs - self.dt * self.b[stage] * self.conv_term(self.V, self.ux, self.uz)
        if self.c[stage] != 0:
            rhs = rhs - self.dt * self.c[stage] * self.conv_term(self.V, self.ux_old, self.uz_old)
        rhs = rhs + self.dt * self.a[stage] * That
        if self.beta != 1.0:
            rhs = rhs + self._explicit_diffusion(self.V, self.nu, stage)
        self._helmholtz(self.solver_V[stage], rhs, self.V)

    def update_T(self, stage):
        rhs = -self.dt * self.b[stage] * self.conv_term(self.T, self.ux, self.uz, add_bc=self.uz * self.dTbcdz1)
        if self.c[stage] != 0:
            rhs = rhs - self.dt * self.c[stage] * self.conv_term(self.T, self.ux_old, self.uz_old,
                                                                 add_bc=self.uz_old * self.dTbcdz1)
        rhs = rhs + self.dt * self.a[stage] * self.kappa * self.dTbcdz2
        if self.beta != 1.0:
            rhs = rhs + self._explicit_diffusion(self.T, self.kappa, stage)
        self._helmholtz(self.solver_T[stage], rhs, self.T)

    def update_P(self, div, singular=True):
        rhs = self.solver_P.solve_rhs(div)
        self.P.vhat = self.solver_P.solve_lhs(rhs)
        if singular:
            self.P.vhat[0, 0] = 0

    def update_pres(self, div, stage):
        self.pres.vhat = self.pres.vhat - 1.0 * self.nu * div * self.beta
        self.pres.vhat = self.pres.vhat + 1.0 / (self.dt * self.a[stage]) * galerkin_to_cheby(self.P.vhat, self.P)

    def _autograd_records(self):
        return torch.is_grad_enabled() and any(getattr(self, k).vhat.requires_grad
                                               for k in ("T", "U", "V", "P", "pres"))

    def update(self, fused=None):
        """One time step (rbc2d.py:396-434).  ``fused=None``: the fused step (``fused()``; the same
        operators regrouped by axis, equal to the plain path to rounding) unless autograd records
        through the state, then the plain path; ``fused=False``: the plain path, operation by
        operation (``update_plain``)."""
        if fused is None:
            fused = not self._autograd_records()
        if fused:
            self.fused().step()
        else:
            self.update_plain()

    def update_plain(self):
        """One time step operation by operation, as the reference runs it (rbc2d.py:396-434)."""
        self.ux_old, self.uz_old = 0, 0
        for rk in range(self.nstage):
            That = galerkin_to_cheby(self.T.vhat, self.T) + self.Tbc_cheby
            if self.dealias:
                self.ux = self.U.dealias.backward(self.U.vhat)
                self.uz = self.V.dealias.backward(self.V.vhat)
            else:
                self.ux = self.U.backward(self.U.vhat)
                self.uz = self.V.backward(self.V.vhat)
            self.update_U(stage=rk)
            self.update_V(That, stage=rk)
            div = self.divergence_velocity(self.U, self.V)
            self.update_P(div)
            self.update_pres(div, stage=rk)
            self.update_velocity(self.P, self.U, self.V)
            self.update_T(stage=rk)
            self.ux_old, self.uz_old = self.ux, self.uz

    # ---------------------------------------------------------- fused step
    def fused(self):
        """The fused line-program step for this configuration (built once).

        The fused passes update the state tensors in place; if the plain path
        (or the user) rebound ``vhat`` since, the current state is copied in.
        """
        if self._fused is None:
            from .fused import FusedStep
            self._fused = FusedStep(self)
        else:
            self._fused.insts[0].sync_in()
        return self._fused

    def update_fused(self, nsteps=1):
        f = self.fused()
        for _ in range(nsteps):
            f.step()

    def iterate(self, maxtime, callback=True, fused=None):
        """The time loop of integrator.py:14-32 (steps, time, save / callback every ``tsave``).  The
        steps are replays of the fused step's CUDA graph (``fused=None``: whenever autograd is not
        recording through the state), else plain ``update(fused=False)`` steps; both give the
        reference's step."""
        if fused is None:
            fused = not self._autograd_records()
        if not fused:
            return Integrator.iterate(self, maxtime, callback, fused=False)
        f = self.fused()
        if f.graph is None:
            f.capture(1)
        eps = 1e-3 * self.dt
        while (self.time + eps) < maxtime:
            f.step()
            self.update_time()
            if self.tsave is not None and (self.time + eps) % self.tsave < self.dt * 0.5:
                self.save()
                if callback:
                    self.callback()

    # -- snapshots in the reference's layout (rbc2d_base.py:208-228)
    def write(self, filename=None, leading_str="", add_time=True):
        """temp / ux / uy / pres groups with v, vhat; time, x, y, nu, kappa, ra, pr at the root.
        Returns the path written."""
        L = float(self.y[-1] - self.y[0])
        meta = {"nu": self.nu, "kappa": self.kappa, "ra": 1.0 / (self.nu * self.kappa) * L ** 3.0,
                "pr": self.nu / self.kappa}
        return self.field.write(filename=filename, leading_str=leading_str, add_time=add_time, dict=meta)

    def read(self, filename=None, leading_str="", add_time=True):
        """Fields, time, ra and pr from a snapshot; the solver plans are rebuilt for them."""
        meta = {"ra": self.ra, "pr": self.pr}
        self.field.read(filename=filename, leading_str=leading_str, add_time=add_time, dict=meta)
        self.time = self.field.fields[0].t
        self.CONFIG.update({k: float(v) for k, v in meta.items()})
        self.__dict__.update(**self.CONFIG)
        self.set_nu_kappa()
        self.setup_solver()
        self._fused = None

    # -- state as host arrays
    def state(self):
        return {k: to_host(getattr(self, k).vhat) for k in ("T", "U", "V", "P", "pres")}

    def set_temperature_noise(self, seed, amplitude):
        """T.v = amplitude * U(-1, 1) (numpy default_rng(seed)), then T.forward()."""
        noise = amplitude * np.random.default_rng(seed).uniform(-1.0, 1.0, self.shape)
        self.T.v = noise
        self.T.forward()
        return noise
