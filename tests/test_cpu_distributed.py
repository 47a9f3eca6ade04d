"""The multi-GPU path of bench.py on CPU: world_size 2 with the gloo backend.

Instances shard across ranks with no exchange on the data path (weak scaling):
every rank draws its own disjoint slice of the batched workload, and the only
collective is the max over ranks of the timed region.
"""
import os

import pytest


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    specs = bench.workload_specs("c4", 8, rank)
    fake_ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
    total = bench.max_over_ranks(fake_ms)
    out.put((rank, [s[3] for s in specs], [s[0] for s in specs], total,
             bench.aggregate_value(len(specs), world, 10, total)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharding_and_timing():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, seeds0, sizes0, t0, v0), (r1, seeds1, sizes1, t1, v1) = res
    assert seeds0 == list(range(100, 108)) and seeds1 == list(range(108, 116))   # disjoint, seeds 100 + i
    assert t0 == t1 == 150.0                                                      # max over ranks
    assert v0 == v1 == pytest.approx(8 * 2 * 10 / 0.150)
    # rank 0 steps exactly the instances of the single-GPU run (weak scaling)
    import bench
    assert [s[0] for s in bench.workload_specs("c4", 8, 0)] == sizes0
