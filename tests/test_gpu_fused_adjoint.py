"""The fused reverse-mode step (fourteen line-program passes) on the GPU.

One adjoint step is compared with the autograd vector-Jacobian product of the
plain step (whose every operator runs a hand-written transposed kernel):
1e-10 relative.  The checkpointed horizon gradient is compared with the
autograd horizon gradient (1e-9) and with central finite differences of the
fused forward map, h = 1e-6 (1e-6 relative, the path's stated target).
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

KEYS = (("TG", "T"), ("UG", "U"), ("VG", "V"), ("PRES", "pres"))


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    return torch


def _ns(case, shape, **kw):
    from pypde_gb300.navier.rbc2d import NavierStokes
    cfg = dict(ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu", tsave=None)
    cfg.update(kw)
    return NavierStokes(case=case, shape=shape, **cfg)


def _random_state(torch, ns, seed):
    rng = np.random.default_rng(seed)
    ns.set_temperature_noise(seed, 1e-2)
    for F in (ns.U, ns.V):
        F.vhat = torch.as_tensor(1e-2 * rng.uniform(-1, 1, tuple(F.vhat.shape)), device="cuda")
    ns.pres.vhat = torch.as_tensor(1e-2 * rng.uniform(-1, 1, tuple(ns.pres.vhat.shape)), device="cuda")
    return tuple(getattr(ns, k).vhat.clone() for k in ("T", "U", "V", "pres"))


STEP_CASES = [("linear", (33, 33), True), ("rbc", (33, 17), True), ("linear", (24, 20), False),
              ("linear", (65, 33), True), ("zero", (17, 33), True)]


@pytest.mark.parametrize("case,shape,dealias", STEP_CASES, ids=[f"{c[0]}-{c[1][0]}x{c[1][1]}" for c in STEP_CASES])
def test_adjoint_step_vs_autograd(torch, case, shape, dealias):
    from pypde_gb300.navier.adjoint import step
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint
    ns = _ns(case, shape, dealias=dealias)
    X = _random_state(torch, ns, 5)
    rng = np.random.default_rng(6)
    gbar = [torch.as_tensor(rng.standard_normal(tuple(x.shape)), device="cuda") for x in X]
    Xr = [x.clone().requires_grad_(True) for x in X]
    with torch.enable_grad():
        Y = step(ns, Xr)
        ref = torch.autograd.grad(Y, Xr, gbar)
    ns2 = _ns(case, shape, dealias=dealias)
    for (k, f), x in zip(KEYS, X):
        getattr(ns2, f).vhat = x.clone()
    fa = FusedAdjoint([ns2])
    bv = fa.views(fa.bar_arena, keys=("UG", "VG", "TG", "PRES"))[0]
    for (k, _), g in zip(KEYS, gbar):
        bv[k].copy_(g)
    fa.adjoint_step_eager()
    for (k, _), r in zip(KEYS, ref):
        e = rel_err(bv[k].cpu().numpy(), r.cpu().numpy())
        assert e < 1e-10, (k, e)


@pytest.mark.parametrize("split", [False, True], ids=["fused", "per-field"])
@pytest.mark.parametrize("case", ["linear", "rbc"])
def test_adjoint_step_beta_vs_autograd(torch, case, split):
    """beta != 1: the reverse-mode passes with the transposed explicit-diffusion terms (Q3s, Q2e)."""
    from pypde_gb300.navier.adjoint import step
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint
    ns = _ns(case, (33, 33), beta=0.4)
    X = _random_state(torch, ns, 15)
    rng = np.random.default_rng(16)
    gbar = [torch.as_tensor(rng.standard_normal(tuple(x.shape)), device="cuda") for x in X]
    Xr = [x.clone().requires_grad_(True) for x in X]
    with torch.enable_grad():
        Y = step(ns, Xr)
        ref = torch.autograd.grad(Y, Xr, gbar)
    ns2 = _ns(case, (33, 33), beta=0.4)
    for (k, f), x in zip(KEYS, X):
        getattr(ns2, f).vhat = x.clone()
    fa = FusedAdjoint([ns2], split=split)
    assert "Q2e" in [p.name for p in fa.aprogs]
    bv = fa.views(fa.bar_arena, keys=("UG", "VG", "TG", "PRES"))[0]
    for (k, _), g in zip(KEYS, gbar):
        bv[k].copy_(g)
    fa.adjoint_step_eager()
    for (k, _), r in zip(KEYS, ref):
        e = rel_err(bv[k].cpu().numpy(), r.cpu().numpy())
        assert e < 1e-10, (k, e)


def _arena_state(torch, fa, X3s):
    Xa = torch.zeros_like(fa.state_arena)
    for v, X3 in zip(fa.views(Xa), X3s):
        for k, x in zip(("TG", "UG", "VG"), X3):
            v[k].copy_(x)
    return Xa


def test_horizon_gradient_vs_autograd_and_fd(torch):
    from pypde_gb300.navier.adjoint import ResidualObjective, random_directions
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint, HorizonGradient
    H, every = 12, 5
    ns = _ns("linear", (33, 33))
    X = _random_state(torch, ns, 3)[:3]
    J_ref, g_ref = ResidualObjective(ns, H, every).value_and_grad(X)
    fa = FusedAdjoint([_ns("linear", (33, 33))])
    fa.capture(1)
    fa.capture_adjoint()
    hg = HorizonGradient(fa, H, every)
    Xa = _arena_state(torch, fa, [X])
    J, g = hg.value_and_grad(Xa)
    assert abs(float(J[0]) - J_ref) / J_ref < 1e-10
    gv = fa.views(g)[0]
    for k, r in zip(("TG", "UG", "VG"), g_ref):
        e = rel_err(gv[k].cpu().numpy(), r.cpu().numpy())
        assert e < 1e-9, (k, e)
    # central differences of the fused forward map, 3 random unit directions
    dirs = random_directions([x.shape for x in X], 3, seed=21, device="cuda")
    h = 1e-6
    for d in dirs:
        Da = _arena_state(torch, fa, [d])
        fd = (float(hg.value(Xa + h * Da)[0]) - float(hg.value(Xa - h * Da)[0])) / (2 * h)
        ad = float((g * Da).sum())
        assert abs(fd - ad) / abs(ad) < 1e-6, (fd, ad)


def test_batched_horizon_gradient_matches_single(torch):
    """Instances of different sizes / Rayleigh numbers: the batch gives each instance's own gradient."""
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint, HorizonGradient
    specs = [((33, 33), 1e5, 1), ((65, 33), 3e5, 2), ((33, 17), 1e4, 3)]
    H, every = 6, 4
    Xs, singles = [], []
    for shape, ra, seed in specs:
        ns = _ns("linear", shape, ra=ra, dt=0.005)
        Xs.append(_random_state(torch, ns, seed)[:3])
        fa1 = FusedAdjoint([_ns("linear", shape, ra=ra, dt=0.005)])
        hg1 = HorizonGradient(fa1, H, every)
        J1, g1 = hg1.value_and_grad(_arena_state(torch, fa1, [Xs[-1]]))
        singles.append((float(J1[0]), {k: v.clone() for k, v in fa1.views(g1)[0].items()}))
    fa = FusedAdjoint([_ns("linear", s, ra=ra, dt=0.005) for s, ra, _ in specs])
    fa.autotune(reps=1)
    fa.autotune_adjoint(reps=1)
    hg = HorizonGradient(fa, H, every)
    J, g = hg.value_and_grad(_arena_state(torch, fa, Xs))
    for i, (J1, g1) in enumerate(singles):
        assert abs(float(J[i]) - J1) / J1 < 1e-12
        for k, v in fa.views(g)[i].items():
            assert rel_err(v.cpu().numpy(), g1[k].cpu().numpy()) < 1e-11, (i, k)


def test_adjoint_step_vs_oracle_directional_derivative(torch):
    """<g, Phi'(X) d> from the oracle's step (CPU, central differences) against <Phi'(X)^T g, d> on the GPU."""
    from oracle import rbc2d as orb
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint
    shape = (33, 33)
    ns = _ns("linear", shape)
    X = [x.cpu().numpy() for x in _random_state(torch, ns, 8)]
    rng = np.random.default_rng(9)
    d = [rng.standard_normal(x.shape) for x in X]
    g = [rng.standard_normal(x.shape) for x in X]
    ref = orb.NavierStokes(case="linear", shape=shape, ra=1e5, pr=1.0, dt=0.01, dealias=True, tsave=None)

    def phi(sign, h=1e-4):
        ref.That, ref.Uhat, ref.Vhat, ref.pres = [x + sign * h * e for x, e in zip(X, d)]
        ref.update()
        return [ref.That, ref.Uhat, ref.Vhat, ref.pres]

    yp, ym = phi(+1), phi(-1)
    lhs = sum(float((gi * (a - b)).sum()) / 2e-4 for gi, a, b in zip(g, yp, ym))
    fa = FusedAdjoint([ns])
    sv = fa.views(fa.state_arena, keys=("UG", "VG", "TG", "PRES"))[0]
    bv = fa.views(fa.bar_arena, keys=("UG", "VG", "TG", "PRES"))[0]
    for (k, _), x, gi in zip(KEYS, X, g):
        sv[k].copy_(torch.as_tensor(x))
        bv[k].copy_(torch.as_tensor(gi))
    fa.adjoint_step()
    rhs = sum(float((bv[k].cpu().numpy() * di).sum()) for (k, _), di in zip(KEYS, d))
    assert abs(lhs - rhs) / abs(rhs) < 1e-8, (lhs, rhs)


def test_horizon_gradient_forms_agree(torch):
    """Sequential or two-stream reverse sweep, eager or one CUDA graph: the same gradient."""
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint, HorizonGradient
    ns = _ns("linear", (33, 17), ra=2e4)
    X = _random_state(torch, ns, 4)[:3]
    fa = FusedAdjoint([_ns("linear", (33, 17), ra=2e4)])
    Xa = _arena_state(torch, fa, [X])
    out = {}
    for overlap in (False, True):
        for graph in (False, True):
            J, g = HorizonGradient(fa, 9, 4, overlap=overlap, graph=graph).value_and_grad(Xa)
            out[(overlap, graph)] = (float(J[0]), g)
    J0, g0 = out[(False, False)]
    for key, (J, g) in out.items():
        assert abs(J - J0) <= 1e-14 * J0, key
        assert float((g - g0).abs().max() / g0.abs().max()) < 1e-13, key


def test_fused_horizon_autograd_function(torch):
    """FusedHorizon (torch.autograd.Function over the fused passes): a loss written in torch on the
    horizon's output back-propagates through the fused reverse sweep; equals HorizonGradient and the
    autograd gradient of the plain step."""
    from pypde_gb300.navier.adjoint import ResidualObjective
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint, FusedHorizon, HorizonGradient
    H, every = 10, 4
    ns = _ns("linear", (33, 33))
    X = _random_state(torch, ns, 6)[:3]
    J_ref, g_ref = ResidualObjective(ns, H, every).value_and_grad(X)
    fa = FusedAdjoint([_ns("linear", (33, 33))])
    hg = HorizonGradient(fa, H, every)
    Xa = _arena_state(torch, fa, [X]).requires_grad_(True)
    mask = torch.zeros_like(Xa)
    for v in fa.views(mask)[0].values():
        v.fill_(1.0)
    Y = FusedHorizon.apply(Xa, hg)
    J = torch.sqrt((((Y - Xa) * mask) ** 2).sum())
    J.backward()
    assert abs(float(J.detach()) - J_ref) / J_ref < 1e-10
    gv = fa.views(Xa.grad)[0]
    for k, r in zip(("TG", "UG", "VG"), g_ref):
        assert rel_err(gv[k].cpu().numpy(), r.cpu().numpy()) < 1e-9, k
    J2, g2 = hg.value_and_grad(Xa.detach())   # (U, V, T entries only; FusedHorizon also gives d/d pres)
    assert float((g2 - Xa.grad * mask).abs().max() / g2.abs().max()) < 1e-12


def test_horizon_gradient_groups_match_one_batch(torch):
    """HorizonGradientGroups (instance groups replayed on their own streams) gives each instance the
    gradient of the one-batch HorizonGradient."""
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint, HorizonGradient, HorizonGradientGroups
    H, every = 6, 3
    mk = lambda s: _ns("linear", (33, 17), ra=2e4 * (1 + s), dt=0.005)  # noqa: E731
    solvers = [mk(s) for s in range(5)]
    for s, ns in enumerate(solvers):
        _random_state(torch, ns, 30 + s)
    fa = FusedAdjoint([mk(s) for s in range(5)])
    for v, ns in zip(fa.views(fa.state_arena), solvers):
        for k, f in (("TG", "T"), ("UG", "U"), ("VG", "V")):
            v[k].copy_(getattr(ns, f).vhat)
    J1, g1 = HorizonGradient(fa, H, every).value_and_grad(fa.state_arena.clone())
    hgs = HorizonGradientGroups(solvers, H, every, groups=3, tune=False)
    assert len(hgs.parts) == 3
    outs = hgs.value_and_grad(hgs.states())
    torch.cuda.synchronize()
    i = 0
    for (fa_g, _, _), (J, g) in zip(hgs.parts, outs):
        for k in range(len(fa_g.insts)):
            assert abs(float(J[k]) - float(J1[i])) <= 1e-12 * abs(float(J1[i]))
            ref = fa.views(g1)[i]
            for key, v in fa_g.views(g)[k].items():
                assert rel_err(v.cpu().numpy(), ref[key].cpu().numpy()) < 1e-11, (i, key)
            i += 1


@pytest.mark.parametrize("split", [False, True], ids=["fused", "per-field"])
@pytest.mark.parametrize("case,beta", [("linear", 1.0), ("rbc", 1.0), ("linear", 0.5)])
def test_adjoint_step_rk3_vs_autograd(torch, case, beta, split):
    """The reverse three-stage step (stages 0, 1 rerun, stages 2, 1, 0 backward with the velocity
    gradients carried between stages) against the autograd VJP of the plain RK3 step."""
    from pypde_gb300.navier.adjoint import step
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint
    ns = _ns(case, (33, 33), integrator="rk3", beta=beta)
    X = _random_state(torch, ns, 25)
    rng = np.random.default_rng(26)
    gbar = [torch.as_tensor(rng.standard_normal(tuple(x.shape)), device="cuda") for x in X]
    Xr = [x.clone().requires_grad_(True) for x in X]
    with torch.enable_grad():
        Y = step(ns, Xr)
        ref = torch.autograd.grad(Y, Xr, gbar)
    ns2 = _ns(case, (33, 33), integrator="rk3", beta=beta)
    for (k, f), x in zip(KEYS, X):
        getattr(ns2, f).vhat = x.clone()
    fa = FusedAdjoint([ns2], split=split)
    assert fa.nstage == 3 and len(fa.alaunches_st) == 3
    sv = fa.views(fa.state_arena, keys=("UG", "VG", "TG", "PRES"))[0]
    x0 = {k: sv[k].clone() for k in sv}
    bv = fa.views(fa.bar_arena, keys=("UG", "VG", "TG", "PRES"))[0]
    for (k, _), g in zip(KEYS, gbar):
        bv[k].copy_(g)
    fa.adjoint_step_eager()
    for k in sv:                               # the step's input is left in place
        assert torch.equal(sv[k], x0[k]), k
    for (k, _), r in zip(KEYS, ref):
        e = rel_err(bv[k].cpu().numpy(), r.cpu().numpy())
        assert e < 1e-10, (k, e)


def test_horizon_gradient_rk3_vs_autograd_and_fd(torch):
    from pypde_gb300.navier.adjoint import ResidualObjective, random_directions
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint, HorizonGradient
    H, every = 8, 3
    ns = _ns("linear", (33, 33), integrator="rk3")
    X = _random_state(torch, ns, 13)[:3]
    J_ref, g_ref = ResidualObjective(ns, H, every).value_and_grad(X)
    fa = FusedAdjoint([_ns("linear", (33, 33), integrator="rk3")])
    fa.capture(1)
    fa.capture_adjoint()
    hg = HorizonGradient(fa, H, every)
    Xa = _arena_state(torch, fa, [X])
    J, g = hg.value_and_grad(Xa)
    assert abs(float(J[0]) - J_ref) / J_ref < 1e-10
    gv = fa.views(g)[0]
    for k, r in zip(("TG", "UG", "VG"), g_ref):
        assert rel_err(gv[k].cpu().numpy(), r.cpu().numpy()) < 1e-9, k
    for d in random_directions([x.shape for x in X], 2, seed=31, device="cuda"):
        Da = _arena_state(torch, fa, [d])
        fd = (float(hg.value(Xa + 1e-6 * Da)[0]) - float(hg.value(Xa - 1e-6 * Da)[0])) / 2e-6
        ad = float((g * Da).sum())
        assert abs(fd - ad) / abs(ad) < 1e-6, (fd, ad)


def test_horizon_graph_rerecorded_after_retuning(torch):
    """Retuning the batch replaces its launches; the horizon's recorded graphs are recorded again
    (a replay of the old ones would read freed descriptors) and give the same gradient."""
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint, HorizonGradient
    ns = _ns("linear", (33, 17), ra=2e4)
    X = _random_state(torch, ns, 40)[:3]
    fa = FusedAdjoint([_ns("linear", (33, 17), ra=2e4)])
    hg = HorizonGradient(fa, 6, 3)
    Xa = _arena_state(torch, fa, [X])
    J0, g0 = hg.value_and_grad(Xa)
    gen = fa.launch_generation
    fa.autotune(reps=1)
    fa.autotune_adjoint(reps=1)
    assert fa.launch_generation > gen
    J1, g1 = hg.value_and_grad(Xa)
    assert hg.graphs["grad"][1] == fa.launch_generation
    assert abs(float(J1[0]) - float(J0[0])) <= 1e-13 * abs(float(J0[0]))
    assert float((g1 - g0).abs().max() / g0.abs().max()) < 1e-11
