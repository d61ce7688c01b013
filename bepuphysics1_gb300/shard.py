"""Scene sharding over ranks with host-side failure detection.

Many independent scenes (the reference steps many Spaces side by side,
ParallelSpaceTestDemo.cs:24-64) shard by scene: scene i belongs to rank
i mod world, and the data path has no collective.  What the ranks share is
liveness: between rounds of steps each rank publishes the last round it
finished in a key-value store (torch.distributed's TCPStore), or the error it
raised, and before launching round r it waits -- with a deadline -- until
every peer has finished round r - 1.  So a rank that raised is seen by the
others before their next launch, and a rank that stops answering (or never
joined) ends their wait with RankFailure instead of a hang.  Nothing here
waits on the GPU: a round's device work is finished before its key is
written.
"""
from __future__ import annotations

import time
from datetime import timedelta
from typing import Callable, Sequence


class RankFailure(RuntimeError):
    """A peer rank raised, or did not finish a round within the deadline."""

    def __init__(self, rank: int, reason: str):
        self.rank = rank
        super().__init__(f"rank {rank}: {reason}")


def shard(indices: Sequence[int] | int, rank: int, world: int) -> list[int]:
    """The scenes of `rank`: every world-th one, starting at `rank`."""
    items = range(indices) if isinstance(indices, int) else indices
    return [i for k, i in enumerate(items) if k % world == rank]


def open_store(host: str, port: int, rank: int, world: int, timeout_s: float = 10.0):
    """The rendezvous store (rank 0 serves it).  Raises RankFailure when the
    ranks do not all arrive within `timeout_s`."""
    import torch.distributed as dist
    try:
        return dist.TCPStore(host, port, world, rank == 0, timedelta(seconds=timeout_s),
                             wait_for_workers=True)
    except Exception as e:  # a peer never joined: the store's own wait ran out
        raise RankFailure(-1, f"rendezvous of {world} ranks failed: {e}") from e


class ShardedRounds:
    """Rounds of work on this rank's shard, checked against the peers'
    progress before each launch."""

    def __init__(self, store, rank: int, world: int, timeout_s: float = 5.0, poll_s: float = 0.005,
                 prefix: str = "bepugpu"):
        self.store, self.rank, self.world = store, rank, world
        self.timeout_s, self.poll_s, self.prefix = timeout_s, poll_s, prefix
        self.round = 0

    def _key(self, what: str, rank: int) -> str:
        return f"{self.prefix}/{what}/{rank}"

    def check_peers(self, finished: int):
        """Returns once every peer has finished round `finished` (-1: none
        needed); raises RankFailure for a peer that failed or ran out of time."""
        deadline = time.monotonic() + self.timeout_s
        pending = [r for r in range(self.world) if r != self.rank]
        while pending:
            still = []
            for r in pending:
                if self.store.check([self._key("failed", r)]):
                    raise RankFailure(r, self.store.get(self._key("failed", r)).decode())
                done = -1
                if self.store.check([self._key("done", r)]):
                    done = int(self.store.get(self._key("done", r)))
                if done < finished:
                    still.append(r)
            pending = still
            if pending:
                if time.monotonic() > deadline:
                    raise RankFailure(pending[0], f"did not finish round {finished} within {self.timeout_s} s")
                time.sleep(self.poll_s)

    def run(self, work: Callable[[int], object]):
        """Runs round `self.round` of this rank's work after the peers
        finished the previous one; publishes success or the error raised."""
        r = self.round
        self.check_peers(r - 1)
        try:
            out = work(r)
        except BaseException as e:
            self.store.set(self._key("failed", self.rank), f"round {r}: {type(e).__name__}: {e}")
            raise
        self.store.set(self._key("done", self.rank), str(r))
        self.round = r + 1
        return out

    def finish(self):
        """Waits for every peer to finish the last round run here."""
        self.check_peers(self.round - 1)
