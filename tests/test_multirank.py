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


# --------------------------------------------------------------------------
# Sharded stepping and failure detection (bepuphysics1_gb300/shard.py), on
# CPU: the scenes step through the oracle, the ranks are gloo processes.

N_SCENES = 6
ROUNDS = 3


def _scene_set():
    from bepuphysics1_gb300 import scenes
    return [scenes.make_tower(40 + 17 * i, seed=700 + i)[:2] for i in range(N_SCENES)]


def _step_scenes(indices, records, rounds_done):
    """Steps each listed scene one step further through the oracle and
    returns its body records."""
    import numpy as np
    import oracle
    from bepuphysics1_gb300.solver import default_settings
    out = {}
    for i in indices:
        b, m = records[i]
        o = oracle.OracleSpace(default_settings(), b, m)
        o.step(np.float32(1 / 60), 63, rounds_done + 1)
        out[i] = o.get_bodies().tobytes()
        o.close()
    return out


def _shard_rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from bepuphysics1_gb300.shard import ShardedRounds, shard
    records = _scene_set()
    mine = shard(N_SCENES, rank, world)
    rounds = ShardedRounds(dist.distributed_c10d._get_default_store(), rank, world, timeout_s=30.0)
    result = {}
    for _ in range(ROUNDS):
        result = rounds.run(lambda r: _step_scenes(mine, records, r))
    rounds.finish()
    gathered = [None] * world
    dist.all_gather_object(gathered, result)
    if rank == 0:
        union = {}
        for g in gathered:
            union.update(g)
        out["union"] = union
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_step_their_shards_and_match_one_rank():
    """Each rank steps scene i for i mod 2 == rank through ROUNDS rounds; the
    union of the shards equals one rank stepping every scene."""
    single = _step_scenes(range(N_SCENES), _scene_set(), ROUNDS - 1)
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_shard_rank, args=(2, port, out), nprocs=2, join=True)
        union = dict(out["union"])
    assert sorted(union) == list(range(N_SCENES))
    for i in range(N_SCENES):
        assert union[i] == single[i], i


def _failing_rank(rank, world, port, mode, out):
    """Rank 1 raises in round 1 ("raise") or leaves after round 0 without a
    word ("vanish"); rank 0 keeps stepping and must see it before its next
    launch."""
    from bepuphysics1_gb300.shard import RankFailure, ShardedRounds, open_store
    try:
        store = open_store("127.0.0.1", port, rank, world, timeout_s=20.0)
        rounds = ShardedRounds(store, rank, world, timeout_s=2.0)

        def work(r):
            if rank == 1 and r == 1:
                if mode == "raise":
                    raise ValueError("scene 3 diverged")
                os._exit(0)  # gone between steps, nothing in flight, no failure key
            return r

        for _ in range(4):
            rounds.run(work)
        out[rank] = ("finished", None)
    except RankFailure as e:
        out[rank] = ("RankFailure", (e.rank, str(e)))
    except ValueError as e:
        out[rank] = ("raised", str(e))


@pytest.mark.parametrize("mode", ["raise", "vanish"])
def test_peer_failure_is_seen_before_the_next_launch(mode):
    port = _free_port()
    ctx = mp.get_context("spawn")
    with mp.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_failing_rank, args=(r, 2, port, mode, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=60)
            assert not p.is_alive()
        res = dict(out)
    kind, detail = res[0]
    assert kind == "RankFailure" and detail[0] == 1, res
    if mode == "raise":
        assert "scene 3 diverged" in detail[1]
        assert res[1] == ("raised", "scene 3 diverged")
    else:
        assert "did not finish round" in detail[1]
        assert 1 not in res


def _lonely_rank(port, out):
    from bepuphysics1_gb300.shard import RankFailure, open_store
    try:
        open_store("127.0.0.1", port, 0, 2, timeout_s=2.0)
        out[0] = "joined"
    except RankFailure as e:
        out[0] = str(e)


def test_rank_that_never_joins_ends_the_rendezvous():
    port = _free_port()
    ctx = mp.get_context("spawn")
    with mp.Manager() as mgr:
        out = mgr.dict()
        p = ctx.Process(target=_lonely_rank, args=(port, out))
        p.start()
        p.join(timeout=60)
        assert not p.is_alive()
        assert "rendezvous of 2 ranks failed" in out[0]
