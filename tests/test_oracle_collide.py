"""Known-answer tests pinning the oracle's narrow phase.

The reference ships no contact golden vectors, so the restatements of
  BoxBoxCollider.AreBoxesColliding   BoxBoxCollider.cs:1494-2388 (face and edge cases)
  BoxSphereTester.AreShapesColliding BoxSphereTester.cs:23-84
  SphereTester.AreSpheresColliding   SphereTester.cs:22-55
and of the manifold updates (BoxContactManifold.cs:122-196,
SphereContactManifold.cs:55-83) are pinned by closed forms: contact points,
depths, normals and ids of simple configurations, id matching across steps,
the first-contact depth rule of the one-contact manifolds, and the round trip
of the manifold's list order through the records.
"""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300.solver import default_settings

DT = np.float32(1 / 60)


def _body(pos, dynamic=True, quat=(0, 0, 0, 1)):
    b = np.zeros(1, N.BODY_DTYPE)
    b["position"] = pos
    b["orientation"] = quat
    b["inverse_mass"] = 1.0 if dynamic else 0.0
    b["local_inverse_inertia"] = np.diag((6.0, 6.0, 6.0)).reshape(9) if dynamic else 0
    b["is_dynamic"] = int(dynamic)
    b["linear_damping"] = 0.03
    b["angular_damping"] = 0.15
    return b


def _shape(kind, size):
    s = np.zeros(1, N.SHAPE_DTYPE)
    s["type"] = kind
    s["size"][0, :len(size)] = size
    return s


def _pair(a=0, b=1):
    m = np.zeros(1, N.MANIFOLD_DTYPE)
    m["body_a"], m["body_b"] = a, b
    m["flags"] = N.MANIFOLD_ACTIVE | N.MANIFOLD_SOLVER_RULE | N.MANIFOLD_GENERATED
    m["kinetic_friction"] = m["static_friction"] = 0.5
    return m


def _collide(bodies, shapes, manifolds, flags=N.STEP_COLLIDE, steps=1):
    o = oracle.OracleSpace(default_settings(), bodies, manifolds, shapes=shapes)
    o.step(DT, flags, steps)
    m, _ = o.get_constraints()
    o.close()
    return m


def _contacts(m, i=0):
    c = m[i]["contacts"][:m[i]["contact_count"]]
    return c["position"].astype(np.float64), c["normal"], c["penetration_depth"], c["id"]


def test_box_resting_on_box_face_contacts():
    """A unit box 0.01 into a wide static box: A's face is the reference face,
    the four bottom corners of B are the contacts, depth 0.01, normal A -> B."""
    ground = _body((0, -0.5, 0), dynamic=False)
    box = _body((0.25, 0.49, -0.125))
    b = np.concatenate([ground, box])
    sh = np.concatenate([_shape(N.SHAPE_BOX, (5, 0.5, 5)), _shape(N.SHAPE_BOX, (0.5, 0.5, 0.5))])
    m = _collide(b, sh, _pair())
    pos, nrm, depth, ids = _contacts(m)
    assert len(ids) == 4
    corners = {(0.25 + sx * 0.5, -0.125 + sz * 0.5) for sx in (-1, 1) for sz in (-1, 1)}
    assert {(round(p[0], 5), round(p[2], 5)) for p in pos} == {(round(x, 5), round(z, 5)) for x, z in corners}
    np.testing.assert_allclose(pos[:, 1], -0.01, atol=1e-6)
    np.testing.assert_allclose(depth, 0.01, atol=1e-6)
    np.testing.assert_array_equal(nrm, np.tile([0, 1, 0], (4, 1)))
    # B's bottom face (y negative): ids 1+bit+4, bit+4, 1+bit, bit with bit = 0
    assert sorted(ids.tolist()) == [0, 1, 4, 5]


def test_separated_boxes_have_no_contacts_and_friction_resets():
    ground = _body((0, -0.5, 0), dynamic=False)
    box = _body((0, 0.49, 0))
    b = np.concatenate([ground, box])
    sh = np.concatenate([_shape(N.SHAPE_BOX, (5, 0.5, 5)), _shape(N.SHAPE_BOX, (0.5, 0.5, 0.5))])
    m = _collide(b, sh, _pair(), flags=N.STEP_ALL)
    assert m[0]["contact_count"] == 4 and m[0]["contacts"]["penetration_impulse"][:4].sum() > 0
    b2 = b.copy()
    b2["position"][1] = (0, 0.7, 0)  # 0.2 above: the separating axis test returns false
    o = oracle.OracleSpace(default_settings(), b2, m, shapes=sh)
    o.step(DT, N.STEP_COLLIDE, 1)
    m2, _ = o.get_constraints()
    assert m2[0]["contact_count"] == 0
    assert m2[0]["twist_impulse"] == 0 and np.all(m2[0]["sliding_impulse"] == 0)


def test_ids_match_across_steps_and_keep_impulses():
    """A second narrow phase over the same poses matches every contact by id:
    positions, ids and warm-start impulses stay; nothing is added."""
    ground = _body((0, -0.5, 0), dynamic=False)
    box = _body((0.1, 0.48, 0.2))
    b = np.concatenate([ground, box])
    sh = np.concatenate([_shape(N.SHAPE_BOX, (5, 0.5, 5)), _shape(N.SHAPE_BOX, (0.4, 0.5, 0.3))])
    o = oracle.OracleSpace(default_settings(), b, _pair(), shapes=sh)
    o.step(DT, N.STEP_COLLIDE | N.STEP_FORCES | N.STEP_SOLVE, 1)
    m1, _ = o.get_constraints()
    o.step(DT, N.STEP_COLLIDE, 1)
    m2, _ = o.get_constraints()
    o.close()
    assert m1[0]["contact_count"] == 4
    np.testing.assert_array_equal(m1[0]["contacts"]["id"], m2[0]["contacts"]["id"])
    np.testing.assert_array_equal(m1[0]["contacts"]["penetration_impulse"], m2[0]["contacts"]["penetration_impulse"])
    assert np.all(m1[0]["contacts"]["penetration_impulse"][:4] > 0)


def test_edge_on_edge_contact():
    """Two boxes turned 45 degrees about crossing horizontal axes touch edge to
    edge: one contact (or a pair) on the crossing, depth = overlap / 1, normal
    vertical."""
    s = np.sqrt(0.5)
    lower = _body((0, 0, 0), dynamic=False, quat=(0, 0, np.sin(np.pi / 8), np.cos(np.pi / 8)))
    upper = _body((0, 2 * s - 0.02, 0), quat=(np.sin(np.pi / 8), 0, 0, np.cos(np.pi / 8)))
    b = np.concatenate([lower, upper])
    sh = np.concatenate([_shape(N.SHAPE_BOX, (0.5, 0.5, 0.5))] * 2)
    m = _collide(b, sh, _pair())
    pos, nrm, depth, ids = _contacts(m)
    assert 1 <= len(ids) <= 4
    np.testing.assert_allclose(np.abs(nrm[:, 1]), 1.0, atol=1e-5)
    np.testing.assert_allclose(depth, 0.02, atol=2e-4)
    np.testing.assert_allclose(pos[:, 0], 0, atol=1e-4)
    np.testing.assert_allclose(pos[:, 2], 0, atol=1e-4)
    # edge ids are GetEdgeId products: (id1 + 1) * 571 + (id2 + 1) * 577 weighted 2549 / 2857
    assert all(i > 2549 * (571 + 577) for i in ids)


def test_sphere_sphere_closed_form():
    a, b_ = _body((0, 0, 0)), _body((0.6, 0.8, 0))
    b = np.concatenate([a, b_])
    sh = np.concatenate([_shape(N.SHAPE_SPHERE, (0.4,)), _shape(N.SHAPE_SPHERE, (0.7,))])
    m = _collide(b, sh, _pair())
    pos, nrm, depth, ids = _contacts(m)
    assert len(ids) == 1
    np.testing.assert_allclose(depth, 0.1, atol=1e-6)
    np.testing.assert_allclose(nrm[0], (0.6, 0.8, 0), atol=1e-6)
    np.testing.assert_allclose(pos[0], np.array((0.6, 0.8, 0)) * (0.4 / 1.1), atol=1e-6)


def test_first_contact_needs_non_negative_depth():
    """SphereContactManifold: a first contact inside the contact distance but
    apart is not taken; once taken, a contact is kept while apart."""
    b = np.concatenate([_body((0, 0, 0)), _body((1.05, 0, 0))])
    sh = np.concatenate([_shape(N.SHAPE_SPHERE, (0.5,))] * 2)
    m = _collide(b, sh, _pair())
    assert m[0]["contact_count"] == 0
    b2 = b.copy()
    b2["position"][1] = (0.95, 0, 0)
    m2 = _collide(b2, sh, _pair())
    assert m2[0]["contact_count"] == 1
    o = oracle.OracleSpace(default_settings(), b, m2, shapes=sh)  # same contact, now 0.05 apart
    o.step(DT, N.STEP_COLLIDE, 1)
    m3, _ = o.get_constraints()
    o.close()
    assert m3[0]["contact_count"] == 1
    np.testing.assert_allclose(m3[0]["contacts"]["penetration_depth"][0], -0.05, atol=1e-6)


def test_box_sphere_outside_and_inside():
    box = _body((0, 0, 0), dynamic=False)
    sph = _body((0.3, 0.9, -0.2))
    b = np.concatenate([box, sph])
    sh = np.concatenate([_shape(N.SHAPE_BOX, (1.0, 0.5, 1.0)), _shape(N.SHAPE_SPHERE, (0.5,))])
    m = _collide(b, sh, _pair())
    pos, nrm, depth, _ = _contacts(m)
    np.testing.assert_allclose(pos[0], (0.3, 0.5, -0.2), atol=1e-6)
    np.testing.assert_allclose(nrm[0], (0, 1, 0), atol=1e-6)
    np.testing.assert_allclose(depth[0], 0.1, atol=1e-6)
    # centre inside: the face of least penetration (x: 1 - 0.8 = 0.2) gives the normal
    b["position"][1] = (0.8, 0.1, 0.3)
    m = _collide(b, sh, _pair())
    pos, nrm, depth, _ = _contacts(m)
    np.testing.assert_allclose(nrm[0], (1, 0, 0), atol=1e-6)
    np.testing.assert_allclose(depth[0], 0.2 + 0.5, atol=1e-6)


def test_list_order_round_trips_through_records():
    """A box sliding off a small box loses contacts and gains others; an oracle
    rebuilt from the records (contact_order included) continues exactly like
    the uninterrupted one."""
    lower = _body((0, 0, 0), dynamic=False)
    upper = _body((0, 0.99, 0))
    b = np.concatenate([lower, upper])
    b["linear_velocity"][1] = (24.0, 0, 9.0)
    sh = np.concatenate([_shape(N.SHAPE_BOX, (1.0, 0.5, 1.0)), _shape(N.SHAPE_BOX, (0.5, 0.5, 0.5))])
    st = default_settings()
    st["gravity"] = (0, 0, 0)
    flags = N.STEP_COLLIDE | N.STEP_POSITIONS
    full = oracle.OracleSpace(st, b, _pair(), shapes=sh)
    seen_ids, codes = set(), set()
    for _ in range(8):
        full.step(DT, flags, 1)
        m, _ = full.get_constraints()
        codes.add(int(m[0]["contact_order"]))
        seen_ids.update(m[0]["contacts"]["id"][:m[0]["contact_count"]].tolist())
        resumed = oracle.OracleSpace(st, full.get_bodies(), m, shapes=sh)
        full.step(DT, flags, 1)
        resumed.step(DT, flags, 1)
        fm, _ = full.get_constraints()
        rm, _ = resumed.get_constraints()
        resumed.close()
        for f in ("contact_count", "contact_order"):
            np.testing.assert_array_equal(fm[f], rm[f])
        np.testing.assert_array_equal(fm["contacts"], rm["contacts"])
    full.close()
    assert len(seen_ids) > 4  # contacts were replaced on the way
