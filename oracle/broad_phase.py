"""Oracle of the broad phase's pair set -- test infrastructure only.

A numpy float32 restatement of the reference's bounding boxes and overlap
test, evaluated in the reference's operation order:
  BoxShape.GetBoundingBox        BEPUphysics/CollisionShapes/ConvexShapes/BoxShape.cs:149-174
  EntityShape.TransformLocalExtremePoints  BEPUphysics/CollisionShapes/EntityShape.cs:58-63
  SphereShape.GetBoundingBox     BEPUphysics/CollisionShapes/ConvexShapes/SphereShape.cs:75-86
  EntityCollidable.ExpandBoundingBox  BEPUphysics/BroadPhaseEntries/MobileCollidables/EntityCollidable.cs:195-216
  BoundingBox.Intersects         BEPUutilities/BoundingBox.cs:58-66
  default kinematic group NoBroadPhase  BEPUphysics/CollisionRuleManagement/CollisionRules.cs:177
and a brute-force pair search over every pair of shaped bodies.
"""
from __future__ import annotations

import numpy as np

SHAPE_NONE, SHAPE_BOX, SHAPE_SPHERE = 0, 1, 2


def bounding_boxes(bodies, shapes, dt):
    """(lo, hi) float32 arrays of shape (n, 3); rows of bodies without a
    shape are NaN."""
    f32 = np.float32
    n = len(bodies)
    p = bodies["position"].astype(f32)
    q = bodies["orientation"].astype(f32)
    h = shapes["size"].astype(f32)
    t = shapes["type"]
    lo = np.full((n, 3), np.nan, f32)
    hi = np.full((n, 3), np.nan, f32)
    qx, qy, qz, qw = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    qX2, qY2, qZ2 = qx + qx, qy + qy, qz + qz
    XX, YY, ZZ = qX2 * qx, qY2 * qy, qZ2 * qz
    XY, XZ, XW = qX2 * qy, qX2 * qz, qX2 * qw
    YZ, YW, ZW = qY2 * qz, qY2 * qw, qZ2 * qw
    one = f32(1)
    M11, M12, M13 = (one - YY) - ZZ, XY + ZW, XZ - YW          # Matrix3x3.CreateFromQuaternion
    M21, M22, M23 = XY - ZW, (one - XX) - ZZ, YZ + XW
    M31, M32, M33 = XZ + YW, YZ - XW, (one - XX) - YY
    def s(v):  # Math.Sign: -1, 0 or 1 (0 for either zero)
        return np.where(v > 0, f32(1), np.where(v < 0, f32(-1), f32(0))).astype(f32)
    hw, hh, hl = h[:, 0], h[:, 1], h[:, 2]
    ox = ((s(M11) * hw) * M11 + (s(M21) * hh) * M21) + (s(M31) * hl) * M31
    oy = ((s(M12) * hw) * M12 + (s(M22) * hh) * M22) + (s(M32) * hl) * M32
    oz = ((s(M13) * hw) * M13 + (s(M23) * hh) * M23) + (s(M33) * hl) * M33
    off = np.stack([ox, oy, oz], axis=1)
    box = t == SHAPE_BOX
    lo[box] = p[box] - off[box]
    hi[box] = p[box] + off[box]
    sph = t == SHAPE_SPHERE
    r = h[sph, 0][:, None]
    lo[sph] = p[sph] - r
    hi[sph] = p[sph] + r
    if dt > 0:
        v = bodies["linear_velocity"].astype(f32)
        step = (v * f32(dt)) * f32(1)
        grow = v > 0
        hi = np.where(grow, hi + step, hi)
        lo = np.where(grow, lo, lo + step)
    return lo, hi


def overlapping_pairs(bodies, shapes, dt, chunk=2048):
    """Every (a, b), a < b, of shaped bodies whose boxes intersect and that
    are not both kinematic, ascending."""
    lo, hi = bounding_boxes(bodies, shapes, dt)
    shaped = np.flatnonzero(shapes["type"] != SHAPE_NONE)
    dyn = bodies["is_dynamic"] != 0
    L, H, D = lo[shaped], hi[shaped], dyn[shaped]
    out = []
    for s0 in range(0, len(shaped), chunk):
        la, ha, da = L[s0:s0 + chunk, None, :], H[s0:s0 + chunk, None, :], D[s0:s0 + chunk, None]
        sep = (L[None] > ha).any(axis=2) | (la > H[None]).any(axis=2)
        ok = ~sep & (da | D[None])
        ia, ib = np.nonzero(ok)
        ia = ia + s0
        keep = ia < ib
        out.append(np.stack([shaped[ia[keep]], shaped[ib[keep]]], axis=1))
    pairs = np.concatenate(out) if out else np.zeros((0, 2), np.int64)
    pairs = np.sort(pairs, axis=1)
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    return pairs[order].astype(np.int32)
