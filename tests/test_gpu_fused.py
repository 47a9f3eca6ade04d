"""GPU parity of the fused line-program step (single instance, CUDA graph, batches).

Tolerances: 1e-9 relative on states after one step, 1e-8 after many steps and
on Nusselt number / kinetic energy (the path's stated target after 100 steps).
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def NS():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from pypde_gb300.navier.rbc2d import NavierStokes
    return NavierStokes


def oracle_run(case, shape, cfg, seed, amp, nsteps):
    from oracle import rbc2d as orb
    ref = orb.NavierStokes(case=case, shape=shape, pr=1.0, tsave=None, **cfg)
    orb.seeded_temperature(ref, seed, amp)
    for _ in range(nsteps):
        ref.update()
    return ref


def compare(ns, ref, tol):
    st = ns.state()
    for name, arr in (("T", ref.That), ("U", ref.Uhat), ("V", ref.Vhat), ("P", ref.Phat), ("pres", ref.pres)):
        e = rel_err(st[name], arr)
        assert e < tol, (name, e)


CASES = [
    ("linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True)),
    ("linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=False)),
    ("linear", (33, 17), dict(ra=3e4, dt=0.01, dealias=True, aspect=2.0)),
    ("rbc", (33, 33), dict(ra=1e5, dt=0.01, dealias=True)),
    ("zero", (33, 33), dict(ra=1e5, dt=0.01, dealias=True)),
    ("linear", (65, 33), dict(ra=1e6, dt=0.005, dealias=True)),
    ("linear", (40, 24), dict(ra=1e5, dt=0.01, dealias=True)),   # 59, 35: dense DCT fallback
]


@pytest.mark.parametrize("case,shape,cfg", CASES, ids=[f"{c[0]}-{c[1][0]}x{c[1][1]}-{i}" for i, c in enumerate(CASES)])
def test_fused_vs_oracle(NS, case, shape, cfg):
    ns = NS(case=case, shape=shape, pr=1.0, tsave=None, integrator="eu", **cfg)
    ns.set_temperature_noise(7, 1e-2)
    f = ns.fused()
    f.step_eager()
    compare(ns, oracle_run(case, shape, cfg, 7, 1e-2, 1), 1e-9)
    for _ in range(9):
        f.step_eager()
    compare(ns, oracle_run(case, shape, cfg, 7, 1e-2, 10), 1e-8)


def test_fused_c1_100_steps_golden(NS, golden):
    """The 65x65, Ra 1e5, dt 0.01 case: Nu, Nuvol and KE after 100 steps within 1e-8 of the reference."""
    ns = NS(case="linear", shape=(65, 65), ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu", tsave=None)
    ns.set_temperature_noise(0, 1e-3)
    f = ns.fused()
    f.capture(1)
    for _ in range(100):
        f.step()
    st = ns.state()
    for name in ("T", "U", "V", "P", "pres"):
        assert rel_err(st[name], golden[f"rbc_c1_s100_{name}"]) < 1e-8, name
    nu, nuv, ke = golden["rbc_c1_s100_scalars"]
    Nu, Nuv = ns.eval_Nu()
    assert abs(Nu - nu) / abs(nu) < 1e-8
    assert abs(Nuv - nuv) / abs(nuv) < 1e-8
    assert abs(ns.eval_KE() - ke) / abs(ke) < 1e-8


def test_graph_replay_equals_eager(NS):
    import torch
    kw = dict(case="linear", shape=(33, 33), ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu", tsave=None)
    a, b = NS(**kw), NS(**kw)
    a.set_temperature_noise(3, 1e-2)
    b.set_temperature_noise(3, 1e-2)
    fa, fb = a.fused(), b.fused()
    fb.capture(1)
    for _ in range(5):
        fa.step_eager()
        fb.step()
    torch.cuda.synchronize()
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


def test_fused_matches_plain(NS):
    kw = dict(case="rbc", shape=(33, 49), ra=2e5, pr=1.0, dt=0.005, dealias=True, integrator="eu", tsave=None)
    a, b = NS(**kw), NS(**kw)
    a.set_temperature_noise(4, 1e-2)
    b.set_temperature_noise(4, 1e-2)
    for _ in range(5):
        a.update(fused=False)
    b.update_fused(5)
    sa, sb = a.state(), b.state()
    for k in sa:
        assert rel_err(sb[k], sa[k]) < 1e-9, k


def test_batched_heterogeneous(NS):
    """Instances of different sizes and Rayleigh numbers in one batch, each vs its own oracle."""
    from pypde_gb300.navier.fused import FusedBatch
    specs = [((33, 33), 1e4, 100), ((65, 33), 1e5, 101), ((33, 129), 3e6, 102), ((129, 65), 1e7, 103),
             ((65, 65), 5e5, 104)]
    solvers = []
    for shape, ra, seed in specs:
        ns = NS(case="linear", shape=shape, ra=ra, pr=1.0, dt=0.005, dealias=True, integrator="eu", tsave=None)
        ns.set_temperature_noise(seed, 1e-3)
        solvers.append(ns)
    fb = FusedBatch(solvers)
    tuned = fb.autotune(reps=1)
    assert {k.split("#")[0] for k in tuned} == {p.name for p in fb.progs}
    # one launch per size class: P2 (y lines) sees Md in {49, 97, 193}
    assert len(fb.launches[1]) == 3
    fb.capture(1)
    for _ in range(3):
        fb.step()
    for ns, (shape, ra, seed) in zip(solvers, specs):
        ref = oracle_run("linear", shape, dict(ra=ra, dt=0.005, dealias=True), seed, 1e-3, 3)
        compare(ns, ref, 1e-8)


def test_warp_parallel_chains_match_sequential(NS):
    """Every chain sweep in warp-per-chain (scanned) mode gives the one-thread-per-chain result
    to rounding; the 65 x 33 and 129 x 65 instances exercise chains longer than a warp."""
    from pypde_gb300.navier.fused import FusedBatch, _CHAIN_CODES
    specs = [((65, 33), 1e5, 1), ((129, 65), 1e6, 2)]
    outs = []
    for warp in (False, True):
        solvers = []
        for shape, ra, seed in specs:
            ns = NS(case="rbc", shape=shape, ra=ra, pr=1.0, dt=0.005, dealias=True, integrator="eu", tsave=None)
            ns.set_temperature_noise(seed, 1e-3)
            solvers.append(ns)
        fb = FusedBatch(solvers)
        tiles = {}
        for tag, (tb, nt, wc, sd, dm) in fb.tiles().items():
            prog = fb.progs[[p.name for p in fb.progs].index(tag.split("#")[0])]
            chains = any(o.code in _CHAIN_CODES for o in prog.ops)
            tiles[tag] = (tb, max(nt, 256), warp and chains)
        fb._build_launches(tiles)
        assert any(L["wc"] for g in fb.launches for L in g) == warp
        for _ in range(3):
            fb.step_eager()
        outs.append([ns.state() for ns in solvers])
    for a, b in zip(*outs):
        for k in a:
            assert rel_err(b[k], a[k]) < 1e-12, k


def test_joint_and_serial_dct_ops_agree(NS):
    """Multi-slot DCT ops (all slots' lines through each transform phase together) give the
    result of one DCT op per slot to rounding (the one-slot ops of even tiles run in the slots' own
    lines with an odd number of FFT stages, the multi-slot ops in FFT buffers); 97-point lines take
    the folded even path, 28-point lines the paired-line path."""
    from pypde_gb300 import _lib
    from pypde_gb300.navier.fused import FusedBatch, _fft_slots
    specs = [((65, 33), 1e5, 1), ((19, 33), 1e4, 2)]
    outs = []
    for sd in (False, True):
        solvers = []
        for shape, ra, seed in specs:
            ns = NS(case="linear", shape=shape, ra=ra, pr=1.0, dt=0.005, dealias=True, integrator="eu", tsave=None)
            ns.set_temperature_noise(seed, 1e-3)
            solvers.append(ns)
        fb = FusedBatch(solvers)
        assert fb.fft
        tiles = {tag: (tb, nt, wc, sd, dm) for tag, (tb, nt, wc, _, dm) in fb.tiles().items()}
        fb._build_launches(tiles)
        joint = [L for g in fb.launches for L in g if _fft_slots(L["prog"]) > 1]
        assert joint and all(L["sd"] == sd for L in joint)
        in_slot = [L for L in joint if any(L["P"].ops[i].code == _lib.OP["DCT"] and L["P"].ops[i].k & _lib.DCT_SLOT
                                           for i in range(L["P"].nops))]
        assert bool(in_slot) == sd
        for _ in range(3):
            fb.step_eager()
        outs.append([ns.state() for ns in solvers])
    for a, b in zip(*outs):
        for k in a:
            assert rel_err(b[k], a[k]) < 1e-12, k


@pytest.mark.parametrize("dealias", [True, False])
def test_in_slot_dct_vs_oracle(NS, dealias):
    """DCT ops run in the slot's own lines and the spare slot (PGX_DCT_SLOT: one-slot ops, even
    tiles, the FFT stage count made odd -- 96-, 128- and 192-point FFTs change plan, 32-, 48- and
    64-point ones keep theirs) in the CTA-wide form (4 lines, 256 threads) and the warp-local form
    (16 lines, 64 threads): each instance follows its oracle for three steps."""
    from pypde_gb300 import _lib
    from pypde_gb300.navier.fused import FusedBatch
    specs = [((33, 65), 1e4, 100), ((129, 33), 1e5, 101), ((65, 129), 3e6, 102)]
    for tb, nt in ((4, 256), (16, 64)):
        solvers = []
        for shape, ra, seed in specs:
            ns = NS(case="linear", shape=shape, ra=ra, pr=1.0, dt=0.005, dealias=dealias, integrator="eu",
                    tsave=None)
            ns.set_temperature_noise(seed, 1e-3)
            solvers.append(ns)
        fb = FusedBatch(solvers)
        assert fb.fft
        names = [p.name for p in fb.progs]
        tiles = {}
        for tag, tile in fb.tiles().items():
            prog = fb.progs[names.index(tag.split("#")[0])]
            tiles[tag] = (tb, nt, False, True, False) if prog.has_dct else tile
        fb._build_launches(tiles)
        flagged = [L for g in fb.launches for L in g
                   if any(L["P"].ops[i].code == _lib.OP["DCT"] and L["P"].ops[i].k & _lib.DCT_SLOT
                          for i in range(L["P"].nops))]
        dct_launches = [L for g in fb.launches for L in g if L["prog"].has_dct]
        assert flagged and len(flagged) == len(dct_launches)
        for _ in range(3):
            fb.step_eager()
        for ns, (shape, ra, seed) in zip(solvers, specs):
            ref = oracle_run("linear", shape, dict(ra=ra, dt=0.005, dealias=dealias), seed, 1e-3, 3)
            compare(ns, ref, 1e-8)


def test_tensor_core_contractions_match(NS):
    """Launches whose DCT ops run as dense matrices and whose DENSE ops (the DCTs, H_y, Q_y) run on
    the FP64 tensor cores (DMMA) give the FFT / FMA-chain step to rounding, and the oracle."""
    from pypde_gb300.navier.fused import FusedBatch, _has_dense
    specs = [((65, 33), 1e5, 1), ((33, 33), 1e4, 2), ((19, 33), 3e4, 3)]
    outs = []
    for dm in (False, True):
        solvers = []
        for shape, ra, seed in specs:
            ns = NS(case="linear", shape=shape, ra=ra, pr=1.0, dt=0.005, dealias=True, integrator="eu", tsave=None)
            ns.set_temperature_noise(seed, 1e-3)
            solvers.append(ns)
        fb = FusedBatch(solvers)
        tiles = {}
        for gl in fb.launches:
            for gi, L in enumerate(gl):
                use = dm and _has_dense(L["prog"], L["key"][1])
                tiles["%s#%d" % (L["name"], gi)] = (8 if use else L["P"].tb, max(L["P"].nthreads, 256), L["wc"],
                                                    False, use)
        fb._build_launches(tiles)
        assert any(L["dm"] for g in fb.launches for L in g) == dm
        if dm:
            assert all(L["P"].fft_n == 0 for g in fb.launches for L in g if L["dm"])
        for _ in range(3):
            fb.step_eager()
        outs.append([ns.state() for ns in solvers])
    for a, b in zip(*outs):
        for k in a:
            assert rel_err(b[k], a[k]) < 1e-11, k
    for ns, (shape, ra, seed) in zip(solvers, specs):
        ref = oracle_run("linear", shape, dict(ra=ra, dt=0.005, dealias=True), seed, 1e-3, 3)
        compare(ns, ref, 1e-8)


def test_step_host_pipeline_matches_step(NS):
    """FusedBatch.step_host (state in pinned host memory, instance groups on their own streams) and
    a step graph with the instance groups as parallel branches give exactly the one-stream graph step."""
    import torch
    from pypde_gb300.navier.fused import FusedBatch
    specs = [((33, 33), 1e4, 1), ((65, 33), 1e5, 2), ((33, 65), 3e5, 3), ((17, 17), 1e4, 4), ((65, 65), 1e6, 5)]
    runs = []
    for host_mode in (False, True, "branches"):
        solvers = []
        for shape, ra, seed in specs:
            ns = NS(case="linear", shape=shape, ra=ra, pr=1.0, dt=0.005, dealias=True, integrator="eu", tsave=None)
            ns.set_temperature_noise(seed, 1e-3)
            solvers.append(ns)
        fb = FusedBatch(solvers)
        fb.capture(1, groups=3 if host_mode == "branches" else 1)
        if host_mode is True:
            assert fb.host_pipeline(3) >= 2
            host = torch.empty(fb.state_arena.numel(), dtype=torch.float64, pin_memory=True)
            host.copy_(fb.state_arena)
            for i in range(4):
                fb.step_host(host, wait=i == 2)
            torch.cuda.synchronize()
            runs.append(host.clone())
        else:
            for _ in range(4):
                fb.step()
            torch.cuda.synchronize()
            runs.append(fb.state_arena.cpu())
    assert fb.graph_groups >= 2
    assert torch.equal(runs[0], runs[1]) and torch.equal(runs[0], runs[2])


BETA_CASES = [
    ("linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu", beta=0.5), None),
    ("linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu", beta=0.5), False),
    ("rbc", (33, 17), dict(ra=3e4, dt=0.01, dealias=True, integrator="eu", beta=0.3, aspect=2.0), None),
    ("linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="rk3", beta=0.5), None),
    ("zero", (40, 24), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu", beta=0.7), False),
]


@pytest.mark.parametrize("case,shape,cfg,split", BETA_CASES,
                         ids=[f"{c[0]}-{c[1][0]}x{c[1][1]}-{c[2]['integrator']}-{c[3]}" for c in BETA_CASES])
def test_fused_beta_vs_oracle(NS, case, shape, cfg, split):
    """beta != 1 (rbc2d.py:268-283, 390-391): beta-implicit ADI tables and pressure update, the explicit
    diffusion through pass P2e and P3 / P3rs; fused and per-field forms against the oracle."""
    from pypde_gb300.navier.fused import FusedBatch
    ns = NS(case=case, shape=shape, pr=1.0, tsave=None, **cfg)
    ns.set_temperature_noise(9, 1e-2)
    fb = FusedBatch([ns], split=split)
    assert fb.beta and "P2e" in [p.name for p in fb.progs]
    for _ in range(3):
        fb.step_eager()
    compare(ns, oracle_run(case, shape, cfg, 9, 1e-2, 3), 1e-8)


def test_fused_beta_mixed_batch(NS):
    """A batch mixing beta = 1 and beta != 1 instances: each against its own oracle run."""
    from pypde_gb300.navier.fused import FusedBatch
    specs = [((33, 33), 1e5, 1.0, 1), ((65, 33), 3e5, 0.5, 2), ((33, 17), 1e4, 0.25, 3)]
    for split in (False, True):
        solvers = []
        for shape, ra, beta, seed in specs:
            ns = NS(case="linear", shape=shape, ra=ra, pr=1.0, dt=0.005, dealias=True, integrator="eu", beta=beta,
                    tsave=None)
            ns.set_temperature_noise(seed, 1e-3)
            solvers.append(ns)
        fb = FusedBatch(solvers, split=split)
        fb.capture(1)
        for _ in range(3):
            fb.step()
        for ns, (shape, ra, beta, seed) in zip(solvers, specs):
            ref = oracle_run("linear", shape, dict(ra=ra, dt=0.005, dealias=True, beta=beta), seed, 1e-3, 3)
            compare(ns, ref, 1e-8)


def test_fused_beta_golden(NS, golden):
    """The reference's own run with beta = 0.5 (33 x 33, Ra 1e5, dt 0.01, seed 4 noise 1e-2): 5 fused steps."""
    ns = NS(case="linear", shape=(33, 33), ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu", beta=0.5,
            tsave=None)
    ns.set_temperature_noise(4, 1e-2)
    assert rel_err(ns.state()["T"], golden["rbc_beta33_T0"]) < 1e-10
    f = ns.fused()
    f.capture(1)
    for _ in range(5):
        f.step()
    st = ns.state()
    for name in ("T", "U", "V", "P", "pres"):
        assert rel_err(st[name], golden[f"rbc_beta33_s5_{name}"]) < 1e-8, name


RK3_CASES = [("linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True)),
             ("rbc", (33, 17), dict(ra=1e5, dt=0.01, dealias=True)),
             ("zero", (33, 33), dict(ra=1e5, dt=0.01, dealias=True)),
             ("linear", (40, 24), dict(ra=1e5, dt=0.01, dealias=True))]


@pytest.mark.parametrize("case,shape,cfg", RK3_CASES, ids=[f"{c[0]}-{c[1][0]}x{c[1][1]}" for c in RK3_CASES])
def test_fused_rk3_vs_oracle(NS, case, shape, cfg):
    """Three-stage IMEX RK3 (rbc2d_base.py:86-102) as 3 x 11 fused passes against the oracle."""
    from oracle import rbc2d as orb
    ns = NS(case=case, shape=shape, pr=1.0, tsave=None, integrator="rk3", **cfg)
    ns.set_temperature_noise(7, 1e-2)
    f = ns.fused()
    assert f.nstage == 3 and len(f.launches) == 3 * len(f.progs)
    f.step_eager()
    ref = orb.NavierStokes(case=case, shape=shape, pr=1.0, tsave=None, integrator="rk3", **cfg)
    orb.seeded_temperature(ref, 7, 1e-2)
    ref.update()
    compare(ns, ref, 1e-9)
    for _ in range(4):
        f.step_eager()
        ref.update()
    compare(ns, ref, 1e-8)


def test_fused_rk3_golden(NS, golden):
    """The reference's own RK3 run (33 x 33, Ra 1e5, dt 0.01, seed 3 noise 1e-2): 5 fused steps from a graph."""
    ns = NS(case="linear", shape=(33, 33), ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="rk3", tsave=None)
    ns.set_temperature_noise(3, 1e-2)
    assert rel_err(ns.state()["T"], golden["rbc_rk3_33_T0"]) < 1e-10
    f = ns.fused()
    f.capture(1)
    for _ in range(5):
        f.step()
    st = ns.state()
    for name in ("T", "U", "V", "P", "pres"):
        assert rel_err(st[name], golden[f"rbc_rk3_33_s5_{name}"]) < 1e-8, name


def test_iterate_fused_matches_update_loop(NS):
    """NavierStokes.iterate (integrator.py:14-32) on the fused graph step gives the update() loop's state,
    time and callback schedule."""
    out = []
    for fused in (False, True):
        ns = NS(case="linear", shape=(33, 33), ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu", tsave=None)
        ns.set_temperature_noise(3, 1e-2)
        calls = []
        ns.save = lambda: None
        ns.callback = lambda: calls.append(round(ns.time, 8))
        ns.tsave = 0.05
        ns.iterate(0.2, fused=fused)
        assert (ns._fused is not None) == fused
        out.append((ns.state(), ns.time, calls))
    (a, ta, ca), (b, tb, cb) = out
    assert abs(ta - tb) < 1e-12 and ca == cb and len(ca) == 4
    for k in a:
        assert rel_err(b[k], a[k]) < 1e-11, k


def test_snapshot_write_read_continues_the_run(NS, tmp_path):
    """NavierStokes.write / read (rbc2d_base.py:208-228): a solver read from the snapshot of another
    (different Ra / Pr on construction) holds its fields, time, Ra and Pr and steps identically."""
    a = NS(case="linear", shape=(33, 33), ra=3e4, pr=0.7, dt=0.01, dealias=True, integrator="eu", tsave=None)
    a.set_temperature_noise(5, 1e-2)
    a.iterate(0.05)
    path = a.write(filename=str(tmp_path / "snap.h5"))
    b = NS(case="linear", shape=(33, 33), ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu", tsave=None)
    b.read(filename=str(tmp_path / "snap.h5"))
    assert path.startswith(str(tmp_path))
    assert abs(b.ra - 3e4) < 1e-6 * 3e4 and abs(b.pr - 0.7) < 1e-12 and abs(b.time - a.time) < 1e-12
    for k, v in a.state().items():
        if k != "P":
            assert np.array_equal(b.state()[k], v), k
    a.update()
    b.update()
    for k in ("T", "U", "V"):
        assert rel_err(b.state()[k], a.state()[k]) < 1e-12, k
