"""Multi-rank host logic on CPU: world size 2 over gloo.

The path shards independent problems across ranks with no data-path
collective; these tests run the sharding, the max-over-ranks timing and the
report gathering in two real processes (gloo, 127.0.0.1)."""
import os
import socket

import pytest

from imscript_gb300 import dist as sdist


def test_partition_covers_every_problem_once_and_balances():
    from imscript_gb300 import synth
    insts = synth.config3(seed=1, n=40, smin=32, smax=200)
    w = [i.unknowns for i in insts]
    for world in (1, 2, 3, 8):
        shards = sdist.partition(w, world)
        flat = sorted(k for s in shards for k in s)
        assert flat == list(range(len(w)))
        assert len(shards) == world
        if world <= 3:
            assert sdist.imbalance(w, shards) < 1.15
    # deterministic: every rank computes the same assignment
    assert sdist.partition(w, 4) == sdist.partition(list(w), 4)


def test_partition_edge_cases():
    assert sdist.partition([], 3) == [[], [], []]
    assert sdist.partition([5.0], 2) == [[0], []]
    with pytest.raises(ValueError):
        sdist.partition([1.0], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, weights, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = sdist.shard(list(range(len(weights))), weights, rank, world)
        step_ms = 10.0 + 5.0 * rank
        mx = sdist.max_over_ranks(step_ms)
        reports = sdist.gather_to_root({"rank": rank, "problems": mine,
                                        "unknowns": sum(weights[k] for k in mine)})
        q.put((rank, mine, mx, reports))
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_timing_and_reports_over_gloo():
    import torch.multiprocessing as mp
    weights = [100, 80, 75, 60, 30, 30, 10, 5, 1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, weights, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, mine, mx, reports = q.get(timeout=120)
        res[rank] = (mine, mx, reports)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(res[0][0] + res[1][0]) == list(range(len(weights)))
    assert not set(res[0][0]) & set(res[1][0])
    assert res[0][1] == res[1][1] == 15.0          # max over ranks of the step time
    assert res[1][2] is None                        # reports land on rank 0 only
    got = {r["rank"]: r for r in res[0][2]}
    assert got[0]["problems"] == res[0][0] and got[1]["problems"] == res[1][0]
    assert got[0]["unknowns"] + got[1]["unknowns"] == sum(weights)
