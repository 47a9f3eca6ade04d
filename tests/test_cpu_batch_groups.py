"""Host logic of FusedBatch's instance groups (graph branches and the host-memory pipeline),
on stand-in CPU tensors: no kernels run."""
import numpy as np
import pytest
import torch

from pypde_gb300.navier.fused import FusedBatch


class _Inst:
    def __init__(self, arrays, shape=(0, 0)):
        self.arrays = arrays
        self.N, self.M = shape


def fake_batch(sizes, order=None, shapes=None):
    """A FusedBatch shell whose instances' states lie back to back in one arena (UG first), in the
    arena order ``order`` (default: instance order)."""
    arena = torch.zeros(int(sum(sizes)), dtype=torch.float64)
    fb = FusedBatch.__new__(FusedBatch)
    order = list(range(len(sizes))) if order is None else order
    offs, off = [0] * len(sizes), 0
    for k in order:
        offs[k] = off
        off += sizes[k]
    fb.state_arena = arena
    fb.insts = [_Inst({"UG": arena[o:o + n]}, shapes[k] if shapes else (0, 0))
                for k, (o, n) in enumerate(zip(offs, sizes))]
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
        assert r == list(range(r[0], r[-1] + 1)) and o0 == starts[r[0]] and o1 == starts[r[-1] + 1]
    assert parts[0][1] == 0 and parts[-1][2] == fb.state_arena.numel()
    if groups <= len(sizes) // 4:                                  # about equal state per group
        per = [o1 - o0 for _, o0, o1 in parts]
        assert max(per) <= sum(sizes) / len(parts) + max(sizes) + 1


def test_split_groups_one_instance():
    fb = fake_batch([100])
    assert [(list(r), a, b) for r, a, b in fb._split_groups(4)] == [([0], 0, 100)]


@pytest.mark.parametrize("seed", [0, 1])
def test_shape_groups_follow_the_arena(seed):
    """With the states laid out by instance shape (FusedBatch's layout; the instances keep the caller's
    order), "shape" groups are the runs of one shape, each one contiguous slice of the arena, and
    numbered groups follow the arena order."""
    rng = np.random.default_rng(seed)
    shapes = [tuple(int(v) for v in s) for s in rng.choice([33, 65, 129], size=(41, 2))]
    sizes = [5 * a * b for a, b in shapes]
    order = sorted(range(len(shapes)), key=lambda k: shapes[k])
    fb = fake_batch(sizes, order, shapes)
    parts = fb._split_groups("shape")
    assert len(parts) == len(set(shapes))
    assert sorted(i for r, _, _ in parts for i in r) == list(range(len(shapes)))
    end = 0
    for r, o0, o1 in parts:
        assert len({shapes[k] for k in r}) == 1
        assert o0 == end and o1 - o0 == sum(sizes[k] for k in r)
        assert [(fb.insts[k].arrays["UG"].data_ptr() - fb.state_arena.data_ptr()) // 8 for k in r] == \
            list(np.cumsum([o0] + [sizes[k] for k in r[:-1]]))
        end = o1
    assert end == fb.state_arena.numel()
    for groups in (2, 5):
        parts = fb._split_groups(groups)
        assert [i for r, _, _ in parts for i in r] == order       # arena order
        assert parts[0][1] == 0 and parts[-1][2] == fb.state_arena.numel()


@pytest.mark.parametrize("per", [2, 3])
def test_shape_groups_split_per_shape(per):
    """"shapeK": every run of one shape in K contiguous groups of about equal instance counts."""
    rng = np.random.default_rng(per)
    shapes = [tuple(int(v) for v in s) for s in rng.choice([33, 65, 129], size=(40, 2))]
    sizes = [5 * a * b for a, b in shapes]
    order = sorted(range(len(shapes)), key=lambda k: shapes[k])
    fb = fake_batch(sizes, order, shapes)
    parts = fb._split_groups("shape%d" % per)
    assert [i for r, _, _ in parts for i in r] == order
    for shape in set(shapes):
        counts = [len(r) for r, _, _ in parts if shapes[r[0]] == shape]
        assert all(shapes[k] == shape for r, _, _ in parts if shapes[r[0]] == shape for k in r)
        assert len(counts) == min(per, shapes.count(shape)) and max(counts) - min(counts) <= 1
    end = 0
    for r, o0, o1 in parts:
        assert o0 == end and o1 - o0 == sum(sizes[k] for k in r)
        end = o1
