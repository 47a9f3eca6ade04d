"""GPU parity of the benchmark configurations at their stated sizes.

* Large plain RBC (513 x 257, aspect 2, Ra 1e8, dt 1e-3, 3/2 dealiasing, 1000 steps):
  the fused step, replayed from its CUDA graph, against signatures of the reference's
  own run (``tests/golden/golden_large.npz``, made by ``make_golden_large.py``) after
  1, 10, 100 and 1000 steps -- states, Nu, Nuvol and KE to 1e-8 (P and pres: no farther
  than the oracle run on this machine, whose LAPACK eigendecomposition of the Poisson plan
  rounds differently from the fixture machine's).
* Batched RBC: a 32-instance slice (every 8th instance) of the benchmark's
  256-instance batch, with autotuned tiles and the tuned graph branches, 5 steps,
  every instance against its own oracle run to 1e-8.
* Helmholtz (I - 0.01 Laplacian) u = f, Dirichlet bases, 1025 x 1025: ADI plan
  against the oracle (1e-10) and the residual of the ADI-factored operator; the exact
  fast-diagonalisation solve at 257 and 1025 against the oracle and its residual.
* Adjoint: the gradient of J = ||Phi^200(X) - X|| at 129 x 129 (checkpoints every
  20 steps) against central differences (h = 1e-6) on 20 random unit directions, 1e-6.
"""
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    return torch


# ------------------------------------------------------------------ 513 x 257, 1000 steps
def test_large_plain_513x257_1000_steps_vs_reference(torch):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden_large import ASPECT, AMP, DT, FIELDS, RA, SEED, SHAPE, SNAPSHOTS, signature
    from pypde_gb300.navier.rbc2d import NavierStokes
    G = np.load(os.path.join(HERE, "golden", "golden_large.npz"))
    snaps = [s for s in SNAPSHOTS if "c3_s%d_scalars" % s in G.files]
    assert snaps and snaps[-1] == 1000, snaps
    ns = NavierStokes(case="linear", shape=SHAPE, ra=RA, pr=1.0, dt=DT, aspect=ASPECT, dealias=True,
                      integrator="eu", tsave=None)
    ns.set_temperature_noise(SEED, AMP)

    def errors(step, state):
        """{(field, part): error relative to the field's max} for one snapshot."""
        out = {}
        for f in FIELDS:
            got = signature(state[f], f)
            big = float(G["c3_s%d_%s_max" % (step, f)][0])
            for part in ("low", "sub"):
                out[(f, part)] = np.max(np.abs(got[part] - G["c3_s%d_%s_%s" % (step, f, part)])) / big
            out[(f, "max")] = abs(got["max"][0] - big) / big
            # a projection on n standard normal weights: error scale max|a| sqrt(n)
            out[(f, "proj")] = np.max(np.abs(got["proj"] - G["c3_s%d_%s_proj" % (step, f)])) / (
                big * np.sqrt(state[f].size))
        return out

    sig0 = signature(ns.state()["T"], "T")  # the initial state
    assert np.max(np.abs(sig0["sub"] - G["c3_s0_T_sub"])) / G["c3_s0_T_max"][0] < 1e-12
    f = ns.fused()
    f.capture(1)
    done, table = 0, []
    for s in snaps:
        for _ in range(s - done):
            f.step()
        done = s
        torch.cuda.synchronize()
        errs = errors(s, ns.state())
        nu, nuv = ns.eval_Nu()
        ke = ns.eval_KE()
        ref = G["c3_s%d_scalars" % s]
        for name, a, b in (("Nu", nu, ref[0]), ("Nuvol", nuv, ref[1]), ("KE", ke, ref[2])):
            errs[(name, "rel")] = abs(a - b) / abs(b)
        table.append((s, errs))
    for s, errs in table:
        print("step %4d  " % s + "  ".join("%s.%s %.1e" % (k[0], k[1], v) for k, v in sorted(errs.items())))
    # P (and through P / dt the pressure pres) comes out of the Poisson plan, whose eigendecomposition
    # the host LAPACK computes; the fixture's machine and this one round it differently.  The oracle --
    # the reference's algorithm -- run here for one step measures that machine-to-machine difference:
    # P and pres may differ from the fixture by up to twice what the oracle does (at least 1e-8).
    from oracle import rbc2d as orb
    ref = orb.NavierStokes(case="linear", shape=SHAPE, ra=RA, pr=1.0, dt=DT, aspect=ASPECT, dealias=True,
                           integrator="eu", tsave=None)
    orb.seeded_temperature(ref, SEED, AMP)
    ref.update()
    here = errors(1, {"T": ref.That, "U": ref.Uhat, "V": ref.Vhat, "P": ref.Phat, "pres": ref.pres})
    print("oracle, step 1 " + "  ".join("%s.%s %.1e" % (k[0], k[1], v) for k, v in sorted(here.items())))
    tol = {k: max(1e-8, 2.0 * v) if k[0] in ("P", "pres") else 1e-8 for k, v in here.items()}
    bad = [(s, k, v) for s, errs in table for k, v in errs.items() if v >= tol.get(k, 1e-8)]
    assert not bad, bad


# ------------------------------------------------------------------ 256-instance batch, slice
def test_benchmark_batch_slice_tuned_graph_vs_oracle(torch):
    """Every 8th instance of the benchmark's batch (sizes {33, 65, 129} per axis, Ra 1e4..1e7,
    dt 0.005), autotuned tiles and tuned parallel graph branches, 5 graph replays."""
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    from bench import workload_specs
    from oracle import rbc2d as orb
    from pypde_gb300.navier.fused import FusedBatch
    from pypde_gb300.navier.rbc2d import NavierStokes
    specs = workload_specs("c4", 256)[::8]
    solvers = []
    for shape, ra, dt, seed, amp, aspect in specs:
        ns = NavierStokes(case="linear", shape=shape, ra=ra, pr=1.0, dt=dt, aspect=aspect, dealias=True,
                          integrator="eu", tsave=None)
        ns.set_temperature_noise(seed, amp)
        solvers.append(ns)
    fb = FusedBatch(solvers)
    fb.autotune(reps=1)
    fb.tune_groups(reps=3)
    assert len(fb.capture_best(tries=2, reps=2)) == 2   # the kept recording is the one stepped below
    assert fb.graph is not None
    for _ in range(5):
        fb.step()
    torch.cuda.synchronize()
    worst = 0.0
    for ns, (shape, ra, dt, seed, amp, aspect) in zip(solvers, specs):
        ref = orb.NavierStokes(case="linear", shape=shape, ra=ra, pr=1.0, dt=dt, aspect=aspect, dealias=True,
                               integrator="eu", tsave=None)
        orb.seeded_temperature(ref, seed, amp)
        for _ in range(5):
            ref.update()
        st = ns.state()
        for name, arr in (("T", ref.That), ("U", ref.Uhat), ("V", ref.Vhat), ("P", ref.Phat), ("pres", ref.pres)):
            e = rel_err(st[name], arr)
            worst = max(worst, e)
            assert e < 1e-8, (shape, ra, name, e)
    assert worst > 0.0


# ------------------------------------------------------------------ Helmholtz 1025^2
def test_helmholtz_adi_1025(torch):
    """(I - 0.01 Laplacian) u = f, CD x CD, 1025 x 1025, f ~ U(-1,1) (seed 1): ADI plan against the
    oracle, and the ADI-factored operator applied to the solution against the right-hand side."""
    import pypde_gb300 as pg
    from oracle import solver as osv
    from oracle import spectral as sp
    N = 1025
    f = np.random.default_rng(1).uniform(-1, 1, (N, N))
    ref = osv.HholtzADI(("CD", "CD"), (N, N), 0.01)
    x_ref = ref.solve_lhs(ref.solve_rhs(f))
    fld = pg.Field([pg.Base(N, "CD"), pg.Base(N, "CD")])
    sol = pg.solverplan_hholtz2d_adi(fld.xs, lam=0.01)
    x = sol.solve_lhs(sol.solve_rhs(f)).cpu().numpy()
    assert rel_err(x, x_ref) < 1e-10
    S, B, I = sp.stencil("CD", N), sp.B2(N), sp.I2(N)
    A = B @ S - 0.01 * I @ S
    lhs = A @ x @ A.T
    rhs = B @ f @ B.T
    assert np.max(np.abs(lhs - rhs)) / np.max(np.abs(rhs)) < 1e-12


def helmholtz_exact_residual(x, f, N, lam):
    """max |(C_x - lam A_x) X C_y^T - lam C_x X A_y^T - B_x F B_y^T| / max |B_x F B_y^T|: the unsplit
    operator of (I - lam Laplacian) u = f premultiplied by B on both axes, C = B S, A = I S."""
    from oracle import spectral as sp
    S, B, I = sp.stencil("CD", N), sp.B2(N), sp.I2(N)
    C, A = B @ S, I @ S
    lhs = (C - lam * A) @ x @ C.T - lam * C @ x @ A.T
    rhs = B @ f @ B.T
    return np.max(np.abs(lhs - rhs)) / np.max(np.abs(rhs))


@pytest.mark.parametrize("N", [257, 1025])
def test_helmholtz_exact_fast_diagonalisation(torch, N):
    """(I - 0.01 Laplacian) u = f, CD x CD, f ~ U(-1,1) (seed 1), solved without the ADI splitting:
    Plan_Poisson with A = -0.01 I_x S_x, C = B_x S_x, alpha_i = 1 - 0.01 w_i.  Against the oracle's
    same plan to 1e-10; the residual of the unsplit operator is bounded by the accuracy of the host
    eigendecomposition of C_y^-1 A_y (the reference's own, ~1e-10 at 257, ~1e-7 at 1025), so the
    GPU solution must leave no more than the oracle's residual (x 2)."""
    import pypde_gb300 as pg
    from oracle import solver as osv
    f = np.random.default_rng(1).uniform(-1, 1, (N, N))
    ref = osv.HholtzFD(("CD", "CD"), (N, N), 0.01)
    x_ref = ref.solve_lhs(ref.solve_rhs(f))
    fld = pg.Field([pg.Base(N, "CD"), pg.Base(N, "CD")])
    sol = pg.solverplan_hholtz2d_fd(fld.xs, lam=0.01)
    x = sol.solve_lhs(sol.solve_rhs(f)).cpu().numpy()
    assert rel_err(x, x_ref) < 1e-10
    r_gpu, r_ref = helmholtz_exact_residual(x, f, N, 0.01), helmholtz_exact_residual(x_ref, f, N, 0.01)
    assert r_gpu <= 2.0 * r_ref + 1e-14, (r_gpu, r_ref)
    if N <= 257:
        old = np.random.default_rng(2).uniform(-1, 1, (N - 2, N - 2))
        assert rel_err(sol.solve_old(old).cpu().numpy(), ref.solve_old(old)) < 1e-10


# ------------------------------------------------------------------ adjoint gradient at 129^2
def test_adjoint_gradient_129_horizon_200_vs_finite_differences(torch):
    from pypde_gb300.navier.adjoint import random_directions
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint, HorizonGradient
    from pypde_gb300.navier.rbc2d import NavierStokes
    ns = NavierStokes(case="linear", shape=(129, 129), ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu",
                      tsave=None)
    ns.set_temperature_noise(3, 1e-2)
    fa = FusedAdjoint([ns])
    fa.capture(1)
    fa.capture_adjoint()
    hg = HorizonGradient(fa, 200, 20)
    X = fa.state_arena.clone()
    J, g = hg.value_and_grad(X)
    assert float(J[0]) > 0
    shapes = [v.shape for v in fa.views(X)[0].values()]
    h, worst = 1e-6, 0.0
    for d in random_directions(shapes, 20, seed=17, device="cuda"):
        D = torch.zeros_like(X)
        for v, e in zip(fa.views(D)[0].values(), d):
            v.copy_(e)
        fd = (float(hg.value(X + h * D)[0]) - float(hg.value(X - h * D)[0])) / (2 * h)
        ad = float((g * D).sum())
        worst = max(worst, abs(fd - ad) / abs(ad))
    assert worst < 1e-6, worst
