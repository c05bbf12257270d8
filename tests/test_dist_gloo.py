"""The multi-rank host logic on CPU with two gloo ranks: the section
sharding plan and the max-over-ranks timing reduction of bench.py."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, shapes, q):
    import sys

    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from pyseistr_gb300.shard import shard_sections

        mine = shard_sections(shapes, rank, world)
        plans = [None] * world
        dist.all_gather_object(plans, mine)
        tmax = bench.max_over_ranks(10.0 + rank, "cpu")
        q.put((rank, plans, tmax))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_sections_and_reduce_time():
    import multiprocessing as mp

    import workloads

    shapes = workloads.batch2d_shapes(count=37)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, shapes, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    plans0, plans1 = res[0][1], res[1][1]
    assert plans0 == plans1  # every rank computes the same plan
    a, b = plans0
    assert sorted(a + b) == list(range(len(shapes))) and not set(a) & set(b)
    size = [s[0] * s[1] for s in shapes]
    la, lb = sum(size[k] for k in a), sum(size[k] for k in b)
    assert abs(la - lb) <= max(size)  # greedy balance bound
    assert res[0][2] == res[1][2] == 11.0  # max over ranks


def test_shard_plan_single_rank_and_errors():
    from pyseistr_gb300.shard import shard_sections

    shapes = [(10, 4), (3, 3), (8, 8)]
    assert shard_sections(shapes, 0, 1) == [0, 1, 2]
    with pytest.raises(ValueError):
        shard_sections(shapes, 2, 2)
