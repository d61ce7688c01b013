"""Scenes for the simulation-island tests: piles of separate columns whose
bodies may go to sleep (IsAlwaysActive cleared), the ground moved into the
middle of the member list, and a moving ground."""
import numpy as np

from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes


def sleepy_pile(nx=16, ny=4, nz=16, seed=1234, ground_at=None, collide=False):
    """A settled pile of nx * nz columns of ny boxes (one island each), none
    of them always active.  ground_at moves the kinematic ground to that
    member index (bodies keep their order around it)."""
    make = scenes.pile_64k_collide if collide else scenes.pile_64k
    out = make(seed=seed, nx=nx, ny=ny, nz=nz)
    b, m, j = out[:3]
    b = b.copy()
    b["activity"] &= ~np.uint32(N.BODY_ALWAYS_ACTIVE)
    rest = tuple(out[3:])
    if ground_at is not None:
        order = list(range(1, len(b)))
        order.insert(ground_at, 0)
        order = np.array(order)
        b, m, j = permute_bodies(b, m, j, order)
        rest = tuple(r[order].copy() for r in rest)  # the shapes, one per body
    return (b, m, j) + rest


def permute_bodies(b, m, j, order):
    """Bodies in the order `order` (new index k holds old body order[k]), the
    constraints' body indices mapped along."""
    new_of = np.empty(len(order), np.int64)
    new_of[order] = np.arange(len(order))
    b = b[order].copy()
    m = m.copy()
    for f in ("body_a", "body_b"):
        v = m[f].astype(np.int64)
        m[f] = np.where(v >= 0, new_of[np.maximum(v, 0)], v)
    if j is not None and len(j):
        j = j.copy()
        for f in ("body_a", "body_b"):
            v = j[f].astype(np.int64)
            j[f] = np.where(v >= 0, new_of[np.maximum(v, 0)], v)
    return b, m, j


def with_moving_kinematics(b, speed=0.5):
    """The kinematic bodies given a horizontal velocity (and their time flag
    reset, as Entity.LinearVelocity's setter does through Activate)."""
    b = b.copy()
    kin = b["is_dynamic"] == 0
    b["linear_velocity"][kin] = (speed, 0.0, 0.0)
    b["velocity_time_below_limit"][kin] = -1.0
    return b
