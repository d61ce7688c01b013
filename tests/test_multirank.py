"""The N > 1 host path on CPU: two gloo ranks shard the many-scene workloads
by scene (scene i on rank i mod N, no collective on the data path) and
combine their results with the reductions bench.py uses (sum of scene-steps,
max of time)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    mine = bench.batch_records(24, rank, world)
    bodies = torch.tensor([float(sum(len(b) for b, _ in mine))], dtype=torch.float64)
    scenes = torch.tensor([float(len(mine))], dtype=torch.float64)
    t = torch.tensor([1.0 + rank], dtype=torch.float64)  # a rank's time
    dist.all_reduce(bodies)
    dist.all_reduce(scenes)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    out[rank] = (bodies.item(), scenes.item(), t.item())
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_scenes():
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    import bench
    whole = bench.batch_records(24)
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    total_bodies = float(sum(len(b) for b, _ in whole))
    for r in (0, 1):
        assert res[r][0] == total_bodies
        assert res[r][1] == 24.0
        assert res[r][2] == 2.0
    # the shards are disjoint and cover every scene
    a = bench.batch_records(24, 0, 2)
    b = bench.batch_records(24, 1, 2)
    assert len(a) + len(b) == len(whole)
    assert all((x[0] == y[0]).all() for x, y in zip(a, whole[0::2]))
    assert all((x[0] == y[0]).all() for x, y in zip(b, whole[1::2]))
