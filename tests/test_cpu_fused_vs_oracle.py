"""The fused step's line programs, run by the NumPy interpreter emulator, against the oracle's step.

For one instance the programs of the fused step (every pass, in launch order, every RK3 stage)
are run on host arrays with the instance's own operator tables, and the state after one step is
compared with ``oracle.rbc2d.NavierStokes.update()`` from the same state.  This checks on the CPU
that the passes, tables and parameters together are the reference's time step; the GPU tests
check the kernels against the same oracle.  The reverse-mode passes are checked the same way
against central differences of the oracle's step.
"""
import numpy as np
import pytest

from line_program_emulator import Machine
from oracle import rbc2d as orb
from pypde_gb300.host import pseudoinverse_d2, stencil_matrix
from pypde_gb300.navier.fused import (build_programs, global_tables_host, host_tables, instance_params,
                                      scratch_shapes)
from pypde_gb300.navier.fused_adjoint import adjoint_shapes, build_adjoint_programs
from pypde_gb300.templates import poisson2d_matrices

# fused state array -> oracle attribute
STATE = {"UG": "Uhat", "VG": "Vhat", "TG": "That", "PG": "Phat", "PRES": "pres"}


def machine_for(ns, split=False, adjoint=False):
    """Emulator machine of the oracle solver ``ns`` (its parameters, tables, boundary lift, state)
    and the programs of the fused (``split`` False) or per-field form of the step; ``adjoint``:
    with the reverse-mode arrays and tables, and the reverse-mode programs."""
    N, M = ns.pres.shape
    tk, beta = ns.Tsp.keys[0], float(ns.beta)
    lens, par = instance_params(N, M, ns.dealias, ns.dt, ns.nu, ns.kappa, ns.scale, beta=beta)
    Nd, Md = lens[5], lens[6]

    def mats(n):
        return stencil_matrix("CN", n), pseudoinverse_d2(n)[2:, :], np.eye(n)[2:, :]

    fd = poisson2d_matrices(mats(N), mats(M), True, ns.scale)
    tables = global_tables_host()
    tables.update(host_tables(N, M, tk, ns.dt * beta, ns.nu, ns.kappa, ns.scale, fd, adjoint=adjoint))
    arrays = {k: np.zeros(s) for k, s in scratch_shapes(N, M, Nd, Md, beta != 1.0).items()}
    if adjoint:
        arrays.update({k: np.zeros(s) for k, s in adjoint_shapes(N, M, Nd, Md, beta != 1.0).items()})
    for k, attr in STATE.items():
        arrays[k] = np.array(getattr(ns, attr), dtype=np.float64)
    arrays["TBCC"] = np.array(ns.Tbc_cheby)
    arrays["DTB1"] = np.array(ns.dTbcdz1)
    arrays["DTB2"] = np.array(ns.dTbcdz2)
    if adjoint:
        for k, attr in STATE.items():
            arrays["b" + k] = np.zeros_like(arrays[k])
    m = Machine(arrays, tables, lens, par)
    stages = [(par, {}, {})]
    if ns.nstage == 3:
        for k in ("UX_A", "UX_B", "UZ_A", "UZ_B"):
            arrays[k] = np.zeros((Nd, Md))
        stages = []
        for st in range(3):
            a, b, c = float(ns.a[st]), float(ns.b[st]), float(ns.c[st])
            spar = instance_params(N, M, ns.dealias, ns.dt, ns.nu, ns.kappa, ns.scale, a, b, c, beta)[1]
            ht = host_tables(N, M, tk, ns.dt * a * beta, ns.nu, ns.kappa, ns.scale, fd)
            cur, old = ("A", "A") if st == 0 else (("B", "A") if st == 1 else ("A", "B"))
            alias = {"UXC": "UX_" + cur, "UZC": "UZ_" + cur, "UXO": "UX_" + old, "UZO": "UZ_" + old}
            stages.append((spar, {k: ht[k] for k in ("Ax_U", "Ax_T", "Ay_U", "Ay_T")}, alias))
    if adjoint:
        return m, stages, build_adjoint_programs(tk, True, split, beta != 1.0)
    return m, stages, build_programs(tk, True, rk3=ns.nstage == 3, split=split, beta=beta != 1.0)


def emulated_step(m, stages, progs):
    for spar, stab, alias in stages:
        m.par = list(spar)
        m.tables.update(stab)
        for name, target in alias.items():
            m.arrays[name] = m.arrays[target]
        for p in progs:
            m.run(p)


CASES = [
    ("linear", (13, 11), dict(dealias=True, integrator="eu", beta=1.0, aspect=1.5)),
    ("linear", (12, 14), dict(dealias=False, integrator="eu", beta=1.0, aspect=1.0)),
    ("rbc", (13, 13), dict(dealias=True, integrator="eu", beta=1.0, aspect=2.0)),
    ("zero", (11, 12), dict(dealias=True, integrator="eu", beta=1.0, aspect=1.0)),
    ("linear", (13, 11), dict(dealias=True, integrator="eu", beta=0.5, aspect=1.0)),
    ("linear", (12, 13), dict(dealias=True, integrator="rk3", beta=1.0, aspect=1.0)),
    ("rbc", (11, 13), dict(dealias=True, integrator="rk3", beta=0.6, aspect=1.5)),
]


@pytest.mark.parametrize("split", [False, True], ids=["fused", "per-field"])
@pytest.mark.parametrize("case,shape,opts", CASES,
                         ids=["%s%dx%d-%s%s-b%g" % (c, s[0], s[1], o["integrator"], "" if o["dealias"] else "-nd",
                                                     o["beta"]) for c, s, o in CASES])
def test_emulated_fused_step_equals_oracle_step(case, shape, opts, split):
    ns = orb.NavierStokes(case=case, shape=shape, ra=3e4, pr=1.0, dt=0.01, tsave=None, **opts)
    orb.seeded_temperature(ns, 4, 5e-2)
    for _ in range(2):   # nonzero velocities and pressure
        ns.update()
    m, stages, progs = machine_for(ns, split)
    ns.update()
    emulated_step(m, stages, progs)
    for k, attr in STATE.items():
        ref = np.asarray(getattr(ns, attr))
        scale = max(np.abs(ref).max(), 1e-300)
        err = np.abs(m.arrays[k] - ref).max() / scale
        assert err < 1e-10, (k, err)


@pytest.mark.parametrize("split", [False, True], ids=["fused", "per-field"])
@pytest.mark.parametrize("case,shape,opts", [c for c in CASES if c[2]["integrator"] == "eu"],
                         ids=["%s%dx%d%s-b%g" % (c, s[0], s[1], "" if o["dealias"] else "-nd", o["beta"])
                              for c, s, o in CASES if o["integrator"] == "eu"])
def test_emulated_reverse_mode_step_is_the_oracle_steps_transpose(case, shape, opts, split):
    """<g, dPhi(X) d> with Phi the oracle's step (central differences: the IMEX Euler step is quadratic
    in the state, so they are exact up to rounding) equals <dPhi(X)^T g, d> from the emulated
    reverse-mode passes."""
    import copy
    ns = orb.NavierStokes(case=case, shape=shape, ra=3e4, pr=1.0, dt=0.01, tsave=None, **opts)
    orb.seeded_temperature(ns, 5, 5e-2)
    for _ in range(2):
        ns.update()
    rng = np.random.default_rng(11)
    keys = ("UG", "VG", "TG", "PRES")     # the step's inputs (the pressure correction is an output)
    X = {k: np.array(getattr(ns, STATE[k]), dtype=np.float64) for k in keys}
    d = {k: 1e-2 * rng.standard_normal(X[k].shape) for k in keys}
    g = {k: rng.standard_normal(np.shape(getattr(ns, STATE[k]))) for k in STATE}
    g["PG"][...] = 0.0     # the pressure correction is scratch of the step: no gradient flows from it

    def phi(Y):
        o = copy.deepcopy(ns)
        for k in keys:
            setattr(o, STATE[k], Y[k].copy())
        o.update()
        return {k: np.asarray(getattr(o, STATE[k])) for k in STATE}

    h = 1e-3
    yp = phi({k: X[k] + h * d[k] for k in keys})
    ym = phi({k: X[k] - h * d[k] for k in keys})
    terms = [g[k] * (yp[k] - ym[k]) / (2 * h) for k in STATE]
    lhs = sum(float(t.sum()) for t in terms)
    m, _, aprogs = machine_for(ns, split, adjoint=True)
    for k in STATE:
        m.arrays["b" + k][...] = g[k]
    for p in aprogs:
        m.run(p)
    rhs = sum(float((m.arrays["b" + k] * d[k]).sum()) for k in keys)
    scale = sum(float(np.abs(t).sum()) for t in terms)
    assert abs(lhs - rhs) <= 1e-9 * scale, (lhs, rhs, scale)
