"""Rayleigh-Benard IMEX time step restated in NumPy (oracle, test infrastructure).

Reference: navier/rbc2d.py (NavierStokes), navier/rbc2d_base.py
(NavierStokesBase, eval_Nu, eval_Nuvol), pypde/field.py (FieldBC).
Supports case "linear" / "zero" / "rbc", integrator "eu" / "rk3", any beta,
dealias on/off.  State lives in ``That``, ``Uhat``, ``Vhat``, ``Phat``, ``pres``.
"""
import numpy as np

from . import spectral as sp
from . import field as fo
from . import solver as so

CONFIG = {"shape": (50, 50), "ra": 5e3, "pr": 1.0, "dt": 0.2, "ndim": 2, "tsave": 0.1,
          "dealias": True, "integrator": "eu", "beta": 1.0, "aspect": 1.0}


def transfer_function(TL, TM, TR, x, k=0.01):
    """transfer_function (rbc2d.py:437-446)."""
    arr = np.zeros(x.shape)
    L = x[-1] - x[0]
    for i in range(x.size):
        xs = x[i] * 2.0 / L
        if xs < 0:
            arr[i] = -k * xs / (k + xs + 1) * (TL - TM) + TM
        else:
            arr[i] = k * xs / (k - xs + 1) * (TR - TM) + TM
    return arr


class NavierStokes:
    """NavierStokes (rbc2d.py:28-434) with NavierStokesBase (rbc2d_base.py:24-114)."""

    def __init__(self, case="rbc", **kwargs):
        if case not in ("rbc", "linear", "zero"):
            raise ValueError("Specified case is not available: ", ["rbc", "linear", "zero"])
        self.case = case
        cfg = dict(CONFIG)
        cfg.update(kwargs)
        self.CONFIG = cfg
        self.__dict__.update(cfg)
        # set_nu_kappa, normalize=True (rbc2d_base.py:68-81)
        self.nu = np.sqrt(self.pr / (self.ra / 1.0 ** 3.0))
        self.kappa = np.sqrt(1 / self.pr / (self.ra / 1.0 ** 3.0))
        self.scale = (self.aspect * 0.5, 0.5)
        N, M = self.shape
        self.deriv = fo.Space2D(("CH", "CH"), (N, M))
        self.x = self.deriv.x(0) * self.scale[0]
        self.y = self.deriv.x(1) * self.scale[1]
        side = "CN" if case == "rbc" else "CD"
        self.Tsp = fo.Space2D((side, "CD"), (N, M))
        self.Usp = fo.Space2D(("CD", "CD"), (N, M))
        self.Psp = fo.Space2D(("CN", "CN"), (N, M))
        self.That = np.zeros(self.Tsp.M)
        self.Uhat = np.zeros(self.Usp.M)
        self.Vhat = np.zeros(self.Usp.M)
        self.Phat = np.zeros(self.Psp.M)
        self.pres = np.zeros((N, M))
        self.time = 0.0
        self.setup_solver()
        if case == "zero":
            self.set_temp_fieldbc_zero()
        else:
            self.set_temp_fieldbc_linear()

    # rbc2d_base.py:86-114
    def _coefficients(self):
        if self.integrator == "rk3":
            self.nstage = 3
            self.a = np.array([8.0 / 15.0, 2.0 / 15.0, 1.0 / 3.0])
            self.b = np.array([8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0])
            self.c = np.array([0, -17.0 / 60.0, -5.0 / 12.0])
        else:
            self.nstage = 1
            self.a = np.array([1.0])
            self.b = np.array([1.0])
            self.c = np.array([0])

    def setup_solver(self):
        """setup_solver (rbc2d.py:180-211)."""
        self._coefficients()
        N, M = self.shape
        self.solver_U, self.solver_V, self.solver_T = [], [], []
        for rk in range(self.nstage):
            lam_u = self.dt * self.a[rk] * self.beta * self.nu
            lam_t = self.dt * self.a[rk] * self.beta * self.kappa
            self.solver_U.append(so.HholtzADI(self.Usp.keys, (N, M), lam_u, self.scale))
            self.solver_V.append(so.HholtzADI(self.Usp.keys, (N, M), lam_u, self.scale))
            self.solver_T.append(so.HholtzADI(self.Tsp.keys, (N, M), lam_t, self.scale))
        self.solver_P = so.Poisson2D(self.Psp.keys, (N, M), singular=True, scale=self.scale)

    def _set_fieldbc(self, bc, axis):
        """FieldBC(T.xs, axis).add_bc(bc) (field.py:359-414) and the derived terms
        dTbcdz2, dTbcdz1, Tbc_cheby (rbc2d.py:135-178)."""
        N, M = self.shape
        keys = ["CH", "CH"]
        keys[axis] = "DC" if self.Tsp.keys[axis] == "CD" else "NC"
        self.Tbcsp = fo.Space2D(keys, (N, M))
        v = sp.backward(keys[axis], bc, axis, N=self.shape[axis])
        self.Tbc_v = v
        self.Tbc_vhat = self.Tbcsp.forward(v)
        self.dTbcdz2 = fo.grad(self.Tbcsp, self.Tbc_vhat, (0, 2), self.scale)
        vhat = fo.grad(self.Tbcsp, self.Tbc_vhat, (0, 1), self.scale)
        if self.dealias:
            self.dTbcdz1 = self.deriv.dealias_backward(vhat)
        else:
            self.dTbcdz1 = self.deriv.backward(vhat)
        self.Tbc_cheby = fo.galerkin_to_cheby(self.Tbcsp, self.Tbc_vhat)

    def set_temp_fieldbc_linear(self):
        N, M = self.shape
        bc = np.zeros((N, 2))
        bc[:, 0], bc[:, 1] = 0.5, -0.5
        self._set_fieldbc(bc, 1)

    def set_temp_fieldbc_zero(self):
        N, M = self.shape
        bc = np.zeros((2, M))
        bc[0, :] = transfer_function(0.5, 0, -0.5, self.y, k=0.02)
        bc[1, :] = bc[0, :]
        self._set_fieldbc(bc, 0)

    # ---- field helpers -------------------------------------------------
    def grad(self, space, vhat, deriv):
        return fo.grad(space, vhat, deriv, self.scale)

    def backward_vel(self, space, vhat):
        if self.dealias:
            return space.dealias_backward(vhat)
        return space.backward(vhat)

    def conv_term(self, space, vhat, ux, uz, add_bc=None):
        """NavierStokes.conv_term (rbc2d.py:236-250)."""
        return fo.convective_term(space, vhat, ux, uz, self.deriv, add_bc=add_bc,
                                  dealias=self.dealias, scale=self.scale)

    # ---- update_* (rbc2d.py:213-394) -----------------------------------
    def update_velocity(self, Phat):
        dpdx = self.grad(self.Psp, Phat, (1, 0))
        dpdz = self.grad(self.Psp, Phat, (0, 1))
        self.Uhat = self.Uhat - fo.cheby_to_galerkin(self.Usp, dpdx)
        self.Vhat = self.Vhat - fo.cheby_to_galerkin(self.Usp, dpdz)

    def divergence_velocity(self, Uhat, Vhat):
        return self.grad(self.Usp, Uhat, (1, 0)) + self.grad(self.Usp, Vhat, (0, 1))

    def _explicit_diffusion(self, space, vhat, coef, stage):
        r = self.dt * self.a[stage] * (1 - self.beta) * coef * self.grad(space, vhat, (2, 0))
        return r + self.dt * self.a[stage] * (1 - self.beta) * coef * self.grad(space, vhat, (0, 2))

    def update_U(self, stage):
        dpdx = self.grad(self.deriv, self.pres, (1, 0))
        rhs = -self.dt * self.a[stage] * dpdx
        rhs = rhs - self.dt * self.b[stage] * self.conv_term(self.Usp, self.Uhat, self.ux, self.uz)
        if self.c[stage] != 0:
            rhs = rhs - self.dt * self.c[stage] * self.conv_term(self.Usp, self.Uhat, self.ux_old, self.uz_old)
        if self.beta != 1.0:
            rhs = rhs + self._explicit_diffusion(self.Usp, self.Uhat, self.nu, stage)
        s = self.solver_U[stage]
        rhs = s.solve_rhs(rhs) + s.solve_old(self.Uhat)
        self.Uhat = s.solve_lhs(rhs)

    def update_V(self, That, stage):
        dpdz = self.grad(self.deriv, self.pres, (0, 1))
        rhs = -self.dt * self.a[stage] * dpdz
        rhs = rhs - self.dt * self.b[stage] * self.conv_term(self.Usp, self.Vhat, self.ux, self.uz)
        if self.c[stage] != 0:
            rhs = rhs - self.dt * self.c[stage] * self.conv_term(self.Usp, self.Vhat, self.ux_old, self.uz_old)
        rhs = rhs + self.dt * self.a[stage] * That
        if self.beta != 1.0:
            rhs = rhs + self._explicit_diffusion(self.Usp, self.Vhat, self.nu, stage)
        s = self.solver_V[stage]
        rhs = s.solve_rhs(rhs) + s.solve_old(self.Vhat)
        self.Vhat = s.solve_lhs(rhs)

    def update_T(self, stage):
        rhs = -self.dt * self.b[stage] * self.conv_term(self.Tsp, self.That, self.ux, self.uz,
                                                       add_bc=self.uz * self.dTbcdz1)
        if self.c[stage] != 0:
            rhs = rhs - self.dt * self.c[stage] * self.conv_term(
                self.Tsp, self.That, self.ux_old, self.uz_old, add_bc=self.uz_old * self.dTbcdz1)
        rhs = rhs + self.dt * self.a[stage] * self.kappa * self.dTbcdz2
        if self.beta != 1.0:
            rhs = rhs + self._explicit_diffusion(self.Tsp, self.That, self.kappa, stage)
        s = self.solver_T[stage]
        rhs = s.solve_rhs(rhs) + s.solve_old(self.That)
        self.That = s.solve_lhs(rhs)

    def update_P(self, div, singular=True):
        rhs = self.solver_P.solve_rhs(div)
        self.Phat = self.solver_P.solve_lhs(rhs)
        if singular:
            self.Phat[0, 0] = 0

    def update_pres(self, div, stage):
        self.pres = self.pres - 1.0 * self.nu * div * self.beta
        self.pres = self.pres + 1.0 / (self.dt * self.a[stage]) * fo.galerkin_to_cheby(self.Psp, self.Phat)

    def update(self):
        """NavierStokes.update (rbc2d.py:396-434)."""
        self.ux_old, self.uz_old = 0, 0
        for rk in range(self.nstage):
            That = fo.galerkin_to_cheby(self.Tsp, self.That) + self.Tbc_cheby
            self.ux = self.backward_vel(self.Usp, self.Uhat)
            self.uz = self.backward_vel(self.Usp, self.Vhat)
            self.update_U(stage=rk)
            self.update_V(That, stage=rk)
            div = self.divergence_velocity(self.Uhat, self.Vhat)
            self.update_P(div)
            self.update_pres(div, stage=rk)
            self.update_velocity(self.Phat)
            self.update_T(stage=rk)
            self.ux_old, self.uz_old = self.ux, self.uz
        self.time += self.dt

    def iterate_steps(self, nsteps):
        for _ in range(nsteps):
            self.update()

    # ---- diagnostics (rbc2d_base.py:344-386) -----------------------------
    def temperature_physical(self):
        return self.Tsp.backward(self.That) + self.Tbc_v

    def eval_Nu(self):
        """eval_Nu: mean of bottom and top plate Nusselt numbers."""
        T = self.temperature_physical()
        Lz = self.y[-1] - self.y[0]
        That = self.deriv.forward(T)
        dThat = self.deriv.derivative(That, 1, axis=1) / (Lz / 2.0)
        dT = self.deriv.backward(dThat)
        dTavg = fo.avg_x(dT, self.deriv.cell_widths(0))
        return (-dTavg[0] * Lz + -dTavg[-1] * Lz) / 2.0

    def eval_Nuvol(self):
        T = self.temperature_physical()
        V = self.Usp.backward(self.Vhat)
        Lz = self.y[-1] - self.y[0]
        That = self.deriv.forward(T)
        dThat = self.deriv.derivative(That, 1, axis=1) / (Lz / 2.0)
        dT = self.deriv.backward(dThat)
        f = (T * V / self.kappa - dT) * Lz
        return fo.avg_vol(f, self.deriv.cell_widths(0), self.deriv.cell_widths(1))

    def eval_KE(self):
        """Kinetic energy 0.5 * avg_vol(u^2 + v^2) on the physical grid.

        pypde defines no kinetic energy; this uses avg_vol's midpoint weights
        (field_operations.py:179-181) on the non-dealiased grid.
        """
        u = self.Usp.backward(self.Uhat)
        v = self.Usp.backward(self.Vhat)
        return 0.5 * fo.avg_vol(u * u + v * v, self.deriv.cell_widths(0), self.deriv.cell_widths(1))


def seeded_temperature(ns, seed, amplitude):
    """Seeded noise initial condition: T.v = amp * U(-1,1) on the physical grid, then
    T.forward() (Galerkin least-squares projection)."""
    rng = np.random.default_rng(seed)
    v = amplitude * rng.uniform(-1.0, 1.0, ns.shape)
    ns.That = ns.Tsp.forward(v)
    return v
