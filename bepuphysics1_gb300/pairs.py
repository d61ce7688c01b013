"""The narrow phase's pair bookkeeping on the host, over the device broad
phase: a manifold record for each pair bepugpu_broad_phase reports, as the
reference's NarrowPhase keeps a pair handler per broad-phase overlap
(NarrowPhaseSystems/NarrowPhase.cs:143-178 adds one for a new overlap,
:254-332 drops a pair whose bounding boxes no longer overlap).

New pairs get an empty BEPUGPU_MANIFOLD_GENERATED record (the device narrow
phase fills it), with the product blend of the two bodies' friction
(MaterialManager.cs:77-85) and the box first in a box-sphere pair
(BoxSpherePairHandler); sphere-sphere and box-sphere pairs are NONCONVEX, as
their pair handlers' manifold constraints are.  Records of pairs that stay
keep their contacts and impulses; new records go after the kept ones, in
ascending pair order.
"""
from __future__ import annotations

import numpy as np

from . import native as N


def _keys(pairs: np.ndarray) -> np.ndarray:
    lo = np.minimum(pairs[:, 0], pairs[:, 1]).astype(np.int64)
    hi = np.maximum(pairs[:, 0], pairs[:, 1]).astype(np.int64)
    return (lo << 32) | hi


class PairRecords:
    """The manifold list of a scene whose pairs come from the broad phase."""

    def __init__(self, friction: np.ndarray, shapes: np.ndarray, manifolds: np.ndarray | None = None):
        self.friction = np.asarray(friction, np.float32)
        self.shapes = np.asarray(shapes, N.SHAPE_DTYPE)
        self.manifolds = np.zeros(0, N.MANIFOLD_DTYPE) if manifolds is None else manifolds.copy()
        self.keys = (_keys(np.stack([self.manifolds["body_a"], self.manifolds["body_b"]], 1))
                     if len(self.manifolds) else np.zeros(0, np.int64))

    def new_records(self, keys: np.ndarray) -> np.ndarray:
        a = (keys >> 32).astype(np.int32)
        b = (keys & 0xffffffff).astype(np.int32)
        t = self.shapes["type"]
        swap = (t[a] == N.SHAPE_SPHERE) & (t[b] == N.SHAPE_BOX)  # box first
        a, b = np.where(swap, b, a), np.where(swap, a, b)
        m = np.zeros(len(keys), N.MANIFOLD_DTYPE)
        m["body_a"], m["body_b"] = a, b
        sphere = (t[a] == N.SHAPE_SPHERE) | (t[b] == N.SHAPE_SPHERE)
        m["flags"] = (N.MANIFOLD_ACTIVE | N.MANIFOLD_SOLVER_RULE | N.MANIFOLD_GENERATED |
                      np.where(sphere, N.MANIFOLD_NONCONVEX, 0)).astype(np.uint32)
        f = self.friction[a] * self.friction[b]
        m["kinetic_friction"] = f
        m["static_friction"] = f
        return m

    def update(self, pairs: np.ndarray, current: np.ndarray | None = None) -> bool:
        """The records for the reported pairs (an (n, 2) array).  `current`: the
        records as the last steps left them (downloaded), in this object's
        order.  Returns whether the pair set changed."""
        if current is not None:
            self.manifolds = current
        keys = _keys(np.asarray(pairs)) if len(pairs) else np.zeros(0, np.int64)
        keep = np.isin(self.keys, keys)
        fresh = np.setdiff1d(keys, self.keys, assume_unique=True)
        if keep.all() and not len(fresh):
            return False
        self.manifolds = np.concatenate([self.manifolds[keep], self.new_records(fresh)])
        self.keys = np.concatenate([self.keys[keep], fresh])
        return True


def settle(space, records: PairRecords, dt: float, steps: int, flags: int = N.STEP_ALL | N.STEP_COLLIDE,
           on_change=None) -> int:
    """Steps a scene whose pairs come from the broad phase: each step asks the
    device broad phase for the pairs, gives new pairs records and drops the
    records of pairs that ended (bepugpu_upload_constraints, which recolours,
    only when the set changed), then steps with the narrow phase.  Returns
    how many steps changed the pair set.  on_change(records) runs after each
    change, before the upload."""
    changes = 0
    for _ in range(steps):
        pairs = space.broad_phase(dt)
        current = space.download_constraints(records.manifolds.copy())[0] if len(records.manifolds) else None
        if records.update(pairs, current):
            changes += 1
            if on_change is not None:
                on_change(records)
            space.upload_constraints(records.manifolds)
        space.step(dt, flags)
    return changes
