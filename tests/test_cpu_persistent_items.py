"""CPU: the work items of the persistent step (``persistent_items``).

The persistent kernel hands items out in list order and an item waits until its
counter has reached its target.  Deadlock freedom and the step's semantics both
rest on two properties checked here on the launch sets of real batches (Euler,
RK3 stages, per-field form, several steps): every wait is satisfied by the items
listed BEFORE it (exactly: the target equals the number of earlier items that
complete that counter when it is the previous pass of the same instance), and
an item of pass p never runs before all of its instance's pass p - 1 items of the
same step -- nor pass 0 before the previous step's last pass.
"""
import collections

import numpy as np
import pytest

from pypde_gb300.navier import fused as F


def synthetic(rng, ninst, npass):
    per_pass, need = [], np.zeros((ninst, npass), dtype=np.int64)
    for p in range(npass):
        its = []
        for k in rng.permutation(ninst):
            for t in range(int(rng.integers(0, 5))):
                its.append((p, 10 * p + int(k), t, int(k)))
                need[k, p] += 1
        per_pass.append(its)
    return per_pass, need


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("nsteps", [1, 3])
def test_items_wait_only_for_earlier_items(seed, nsteps):
    rng = np.random.default_rng(seed)
    ninst, npass = int(rng.integers(1, 7)), int(rng.integers(1, 12))
    per_pass, need = synthetic(rng, ninst, npass)
    items = F.persistent_items(per_pass, need, nsteps)
    assert len(items) == nsteps * sum(len(x) for x in per_pass)
    done = collections.Counter()
    for prog, desc, tile, wait, nd, ctr in items:
        if wait >= 0:
            # the earlier items already completing the counter reach exactly the target once the
            # whole previous pass (of this step, or of the previous step for pass 0) is done
            assert done[wait] >= nd, (wait, nd, done[wait])
            k, p = divmod(ctr, npass)
            kw, pw = divmod(wait, npass)
            assert kw == k and pw == (p - 1) % npass
        else:
            assert ctr % npass == 0 and nd == 0
        done[ctr] += 1
    # per step: every counter ends at nsteps x need
    for k in range(ninst):
        for p in range(npass):
            assert done[k * npass + p] == nsteps * need[k, p]


def test_items_of_a_pass_wait_for_the_whole_previous_pass():
    # two instances, three passes, one step: instance 0's pass 1 needs all 3 of its pass-0 tiles
    per_pass = [[(0, 0, 0, 0), (0, 0, 1, 0), (0, 1, 0, 1), (0, 0, 2, 0)],
                [(1, 2, 0, 0), (1, 3, 0, 1)],
                [(2, 4, 0, 1), (2, 5, 0, 0)]]
    need = np.array([[3, 1, 1], [1, 1, 1]])
    items = F.persistent_items(per_pass, need, 2)
    first_pass1 = items[4]
    assert first_pass1[3:] == (0, 3, 1)   # waits on counter (0, pass 0) for 3 completions
    second_step_pass0 = items[8]
    assert second_step_pass0[3:] == (2, 1, 0)   # waits on instance 0's last pass of step 0
