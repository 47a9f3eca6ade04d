"""Host logic of FusedBatch's instance groups (graph branches and the host-memory pipeline),
on stand-in CPU tensors: no kernels run."""
import numpy as np
import pytest
import torch

from pypde_gb300.navier.fused import FusedBatch


class _Inst:
    def __init__(self, arrays):
        self.arrays = arrays


def fake_batch(sizes):
    """A FusedBatch shell whose instances' states lie back to back in one arena (UG first)."""
    arena = torch.zeros(int(sum(sizes)), dtype=torch.float64)
    fb = FusedBatch.__new__(FusedBatch)
    fb.state_arena, fb.insts, off = arena, [], 0
    for n in sizes:
        fb.insts.append(_Inst({"UG": arena[off:off + n]}))
        off += n
    return fb


@pytest.mark.parametrize("groups", [1, 2, 3, 4, 8, 300])
@pytest.mark.parametrize("seed", [0, 1])
def test_split_groups_are_contiguous_and_balanced(groups, seed):
    rng = np.random.default_rng(seed)
    sizes = [int(s) ** 2 * 5 for s in rng.choice([33, 65, 129], size=37)]
    fb = fake_batch(sizes)
    parts = fb._split_groups(groups)
    assert 1 <= len(parts) <= min(groups, len(sizes))
    idx = [i for r, _, _ in parts for i in r]
    assert idx == list(range(len(sizes)))                         # every instance once, in order
    starts = np.concatenate([[0], np.cumsum(sizes)])
    for r, o0, o1 in parts:                                       # each group's arena slice is its states
        assert o0 == starts[r.start] and o1 == starts[r.stop]
    assert parts[0][1] == 0 and parts[-1][2] == fb.state_arena.numel()
    if groups <= len(sizes) // 4:                                  # about equal state per group
        per = [o1 - o0 for _, o0, o1 in parts]
        assert max(per) <= sum(sizes) / len(parts) + max(sizes) + 1


def test_split_groups_one_instance():
    fb = fake_batch([100])
    assert [(list(r), a, b) for r, a, b in fb._split_groups(4)] == [([0], 0, 100)]
