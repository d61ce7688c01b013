"""A pile dropped onto the ground and settled with the broad phase, the
narrow phase and the solver, all on the oracle: the pair records follow the
broad phase's pair set (bepuphysics1_gb300/pairs.py) as the reference's
narrow phase follows its overlaps (NarrowPhase.cs:143-178,254-332)."""
import numpy as np

import oracle
from oracle.broad_phase import overlapping_pairs
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.pairs import PairRecords
from bepuphysics1_gb300.solver import default_settings

DT = np.float32(1 / 60)


def test_pair_records_follow_the_pair_set():
    b, shapes, fr = scenes.dropped_pile(nx=2, ny=2, nz=2)
    r = PairRecords(fr, shapes)
    assert r.update(np.array([[0, 1], [0, 2], [1, 2]]))
    np.testing.assert_array_equal(r.manifolds["body_a"], [0, 0, 1])
    assert np.all(r.manifolds["flags"] & N.MANIFOLD_GENERATED)
    np.testing.assert_allclose(r.manifolds["kinetic_friction"][2], fr[1] * fr[2])
    m = r.manifolds.copy()
    m["contact_count"][1] = 3  # the device filled one
    assert not r.update(np.array([[0, 1], [0, 2], [1, 2]]), m)
    assert r.update(np.array([[0, 2], [1, 2], [2, 3]]), m)
    np.testing.assert_array_equal(np.stack([r.manifolds["body_a"], r.manifolds["body_b"]], 1),
                                  [[0, 2], [1, 2], [2, 3]])
    assert r.manifolds["contact_count"][0] == 3  # a kept pair keeps its record


def test_dropped_pile_settles_on_the_oracle():
    b, shapes, fr = scenes.dropped_pile(nx=3, ny=3, nz=3)
    records = PairRecords(fr, shapes)
    s = default_settings()
    bodies, o = b, None
    changes = 0
    for step in range(150):
        pairs = overlapping_pairs(bodies, shapes, DT)
        current = o.get_constraints()[0] if o is not None else None
        if records.update(pairs, current) or o is None:
            changes += 1
            o = oracle.OracleSpace(s, bodies, records.manifolds, shapes=shapes)
        o.step(DT, N.STEP_ALL | N.STEP_COLLIDE)
        bodies = o.get_bodies()
    dyn = bodies["is_dynamic"] == 1
    # every box came down onto its column and the columns stand: low speeds, contacts in place
    assert changes > 3
    assert float(np.abs(bodies["linear_velocity"][dyn]).max()) < 0.5
    assert bodies["position"][dyn][:, 1].max() < 4.0
    m = o.get_constraints()[0]
    assert int(m["contact_count"].sum()) >= 4 * 27
