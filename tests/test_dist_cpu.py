"""Multi-process host logic on CPU (gloo, world size 2): mesh sharding of the
batched form and the max/sum-over-ranks reductions the bench reports with."""
import os
import socket

import numpy as np
import pytest

from nexusbvh_gb300 import dist, scenes


def test_shards_are_disjoint_complete_and_balanced():
    counts = scenes.batch_counts(1024, seed=3)
    for world in (1, 2, 3, 4, 8):
        shards = [dist.shard_meshes(counts, world, r) for r in range(world)]
        allm = np.concatenate(shards)
        assert sorted(allm.tolist()) == list(range(len(counts)))
        loads = [int(counts[s].sum()) for s in shards]
        assert max(loads) - min(loads) <= int(counts.max())
    assert dist.shard_meshes([5, 0, 7], 2, 0).tolist() == [2]
    assert dist.shard_meshes([5, 0, 7], 2, 1).tolist() == [0, 1]
    with pytest.raises(ValueError):
        dist.shard_meshes([1], 2, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as td
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        counts = scenes.batch_counts(64, seed=1)
        mine = dist.shard_meshes(counts, world, rank)
        tris = float(counts[mine].sum())
        elapsed = 0.5 + rank  # rank 1 is the slowest
        rate = dist.whole_job_rate(tris, elapsed)
        out.put((rank, mine.tolist(), dist.max_over_ranks(elapsed), rate))
        td.barrier()
    finally:
        td.destroy_process_group()


def test_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    counts = scenes.batch_counts(64, seed=1)
    assert sorted(res[0][1] + res[1][1]) == list(range(64))
    assert res[0][2] == res[1][2] == 1.5
    assert res[0][3] == pytest.approx(float(counts.sum()) / 1.5)
    assert res[1][3] == pytest.approx(res[0][3])
