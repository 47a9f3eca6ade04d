"""GPU: the persistent step (pgx_run_persistent) -- whole steps of a batch in one launch.

* A heterogeneous batch (sizes 33..129, Ra 1e4..1e7) for 3 steps in one launch
  against the same batch stepped by the per-pass graph (1e-12: the two forms run
  the same programs and tiles, but a CTA size of its own can change the order of
  a few per-line sums) and against the oracle (1e-8); and the same batch as 3
  launches of one step each, replayed from a CUDA graph.
* A single instance in the per-field form (the twelve-pass step) likewise.
* A wait that cannot be satisfied (a target no item reaches) ends the launch after
  its short bounded spin with PGX_PERSIST_TIMEOUT and the item's index, and the
  context stays usable; an item naming a program that does not exist ends it with
  PGX_PERSIST_BAD_ITEM.  No wait runs unbounded and nothing faults.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

SPECS = [((33, 33), 1e4, 100), ((65, 33), 1e5, 101), ((33, 129), 3e6, 102), ((129, 65), 1e7, 103),
         ((65, 65), 5e5, 104)]


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    return torch


def batch(specs, split=None):
    from pypde_gb300.navier.fused import FusedBatch
    from pypde_gb300.navier.rbc2d import NavierStokes
    solvers = []
    for shape, ra, seed in specs:
        ns = NavierStokes(case="linear", shape=shape, ra=ra, pr=1.0, dt=0.005, dealias=True, integrator="eu",
                          tsave=None)
        ns.set_temperature_noise(seed, 1e-3)
        solvers.append(ns)
    return solvers, FusedBatch(solvers, split=split)


def oracle(shape, ra, seed, nsteps):
    from oracle import rbc2d as orb
    ref = orb.NavierStokes(case="linear", shape=shape, ra=ra, pr=1.0, dt=0.005, dealias=True, integrator="eu",
                           tsave=None)
    orb.seeded_temperature(ref, seed, 1e-3)
    for _ in range(nsteps):
        ref.update()
    return ref


@pytest.mark.parametrize("split", [False, True], ids=["fused", "per-field"])
def test_persistent_batch_three_steps_one_launch(torch, split):
    solvers, fb = batch(SPECS, split=split)
    fb.autotune(reps=1)
    init = fb.state_arena.clone()
    fb.capture(1)
    for _ in range(3):
        fb.step()
    torch.cuda.synchronize()
    graph_state = fb.state_arena.clone()
    fb.state_arena.copy_(init)
    info = fb.persistent(nsteps=3)
    assert info["nitems"] > 0 and info["ctas_per_sm"] >= 1
    fb.run_persistent()
    assert fb.persistent_error() == (0, 0)
    assert rel_err(fb.state_arena.cpu().numpy(), graph_state.cpu().numpy()) < 1e-12
    for ns, (shape, ra, seed) in zip(solvers, SPECS):
        ref = oracle(shape, ra, seed, 3)
        st = ns.state()
        for name, arr in (("T", ref.That), ("U", ref.Uhat), ("V", ref.Vhat), ("P", ref.Phat), ("pres", ref.pres)):
            assert rel_err(st[name], arr) < 1e-8, (shape, name)
    # one step per launch, recorded in a graph and replayed three times: the same state
    fb.state_arena.copy_(init)
    fb.persistent(nsteps=1)
    fb.capture_persistent()
    fb.state_arena.copy_(init)
    for _ in range(3):
        fb.step_persistent()
    assert fb.persistent_error() == (0, 0)
    assert rel_err(fb.state_arena.cpu().numpy(), graph_state.cpu().numpy()) < 1e-12


def test_persistent_single_instance_per_field(torch):
    from pypde_gb300.navier.rbc2d import NavierStokes
    ns = NavierStokes(case="linear", shape=(65, 65), ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu",
                      tsave=None)
    ns.set_temperature_noise(0, 1e-3)
    f = ns.fused()
    f.persistent(nsteps=4)
    f.run_persistent()
    assert f.persistent_error() == (0, 0)
    from oracle import rbc2d as orb
    ref = orb.NavierStokes(case="linear", shape=(65, 65), ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu",
                           tsave=None)
    orb.seeded_temperature(ref, 0, 1e-3)
    for _ in range(4):
        ref.update()
    st = ns.state()
    for name, arr in (("T", ref.That), ("U", ref.Uhat), ("V", ref.Vhat), ("P", ref.Phat), ("pres", ref.pres)):
        assert rel_err(st[name], arr) < 1e-8, name


def test_persistent_unsatisfiable_wait_times_out_and_the_context_survives(torch):
    solvers, fb = batch(SPECS[:2])
    init = fb.state_arena.clone()
    fb.persistent(nsteps=1, spin_seconds=1e-3)
    q = fb._persist
    items = q["d_items"].view(-1, 6)
    # the last item waits for a count its counter never reaches: no item adds that many
    last = q["nitems"] - 1
    items[last, 3] = 0
    items[last, 4] = 1 << 30
    fb.run_persistent()
    err, where = fb.persistent_error()
    assert (err, where) == (1, last)   # PGX_PERSIST_TIMEOUT at that item
    # the context is usable: the ordinary step still runs and matches the oracle
    fb.state_arena.copy_(init)
    fb.step_eager()
    torch.cuda.synchronize()
    for ns, (shape, ra, seed) in zip(solvers, SPECS[:2]):
        ref = oracle(shape, ra, seed, 1)
        assert rel_err(ns.state()["T"], ref.That) < 1e-9


def test_persistent_bad_item_is_refused_on_the_device(torch):
    solvers, fb = batch(SPECS[:1])
    fb.persistent(nsteps=1, spin_seconds=1e-3)
    q = fb._persist
    q["d_items"].view(-1, 6)[0, 0] = q["nprogs"] + 7   # a program index past the end
    fb.run_persistent()
    err, where = fb.persistent_error()
    assert err == 2 and where == 0   # PGX_PERSIST_BAD_ITEM
