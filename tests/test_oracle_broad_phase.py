"""Closed-form pins of the oracle's broad phase restatement (the bounding
boxes of BoxShape.cs:149-174 and SphereShape.cs:75-86, the velocity expansion
of EntityCollidable.cs:195-216, BoundingBox.Intersects and the kinematic
NoBroadPhase rule)."""
import numpy as np

from bepuphysics1_gb300 import native as N
from oracle import broad_phase as obp


def _bodies(n):
    b = np.zeros(n, N.BODY_DTYPE)
    b["orientation"] = (0, 0, 0, 1)
    b["is_dynamic"] = 1
    return b


def test_box_and_sphere_boxes():
    b = _bodies(3)
    sh = np.zeros(3, N.SHAPE_DTYPE)
    sh["type"] = (N.SHAPE_BOX, N.SHAPE_BOX, N.SHAPE_SPHERE)
    sh["size"][0] = (1, 2, 3)
    sh["size"][1] = (1, 2, 3)
    sh["size"][2] = (0.5, 0, 0)
    b["position"][1] = (10, 0, 0)
    s = np.float32(np.sqrt(0.5))
    b["orientation"][1] = (0, 0, s, s)  # 90 degrees about z: x and y extents swap
    b["position"][2] = (0, 5, 0)
    lo, hi = obp.bounding_boxes(b, sh, 0.0)
    np.testing.assert_allclose(lo[0], (-1, -2, -3)); np.testing.assert_allclose(hi[0], (1, 2, 3))
    np.testing.assert_allclose(hi[1] - lo[1], (4, 2, 6), atol=1e-6)
    np.testing.assert_allclose(lo[2], (-0.5, 4.5, -0.5)); np.testing.assert_allclose(hi[2], (0.5, 5.5, 0.5))


def test_velocity_expands_the_leading_side_only():
    b = _bodies(1)
    b["linear_velocity"][0] = (3, -6, 0)
    sh = np.zeros(1, N.SHAPE_DTYPE)
    sh["type"] = N.SHAPE_SPHERE
    sh["size"][0] = (1, 0, 0)
    lo, hi = obp.bounding_boxes(b, sh, 0.5)
    np.testing.assert_allclose(lo[0], (-1, -4, -1))  # y grows downwards by |v| dt, z (v = 0) on the min side by 0
    np.testing.assert_allclose(hi[0], (2.5, 1, 1))


def test_pairs_touching_faces_count_and_kinematic_pairs_do_not():
    b = _bodies(4)
    sh = np.zeros(4, N.SHAPE_DTYPE)
    sh["type"] = N.SHAPE_BOX
    sh["size"] = (1, 1, 1)
    b["position"][1] = (2, 0, 0)      # touches body 0 face to face: Intersects is inclusive
    b["position"][2] = (4.01, 0, 0)   # 0.01 short of body 1
    b["position"][3] = (-2, 0, 0)     # touches body 0 on its other side
    b["is_dynamic"][[0, 3]] = 0       # 0 and 3 are kinematic: no pair between them
    pairs = obp.overlapping_pairs(b, sh, 0.0)
    assert pairs.tolist() == [[0, 1]]
    b["is_dynamic"][3] = 1
    assert obp.overlapping_pairs(b, sh, 0.0).tolist() == [[0, 1], [0, 3]]
