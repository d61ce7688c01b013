"""Seeded synthetic workloads (libbepuscenes.so) as numpy record arrays.

The named workloads follow the benchmark configurations:
    pile_1k     1,000 unit boxes (1 kg, friction 0.6) in a 10x10x10 grid at
                1.05 m with +-0.05 m jitter, settled on a 100x1x100 ground.
    pile_64k    65,536 boxes, sizes U(0.5, 1.5) per axis, density 1, friction
                U(0.4, 0.8), 64x16x64 columns at 2.0 m with +-0.1 m jitter.
    tower(n)    one scene of n boxes/spheres (1 m, 1 kg) in towers of 4-32.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native as N


def _collect(handle, with_shapes: bool = False, with_friction: bool = False):
    lib = N.load_scene_library()
    nb, nm, nj = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    lib.bepuscene_counts(handle, ctypes.byref(nb), ctypes.byref(nm), ctypes.byref(nj))
    bodies = np.zeros(nb.value, N.BODY_DTYPE)
    manifolds = np.zeros(nm.value, N.MANIFOLD_DTYPE)
    joints = np.zeros(nj.value, N.JOINT_DTYPE)
    lib.bepuscene_copy(handle, N.ptr(bodies), N.ptr(manifolds), N.ptr(joints))
    shapes = np.zeros(nb.value, N.SHAPE_DTYPE)
    lib.bepuscene_shapes(handle, N.ptr(shapes))
    friction = np.zeros(nb.value, np.float32)
    lib.bepuscene_body_friction(handle, N.ptr(friction))
    lib.bepuscene_free(handle)
    if with_friction:
        return bodies, shapes, friction
    if with_shapes:
        return bodies, manifolds, joints, shapes
    return bodies, manifolds, joints


def make_pile(**overrides):
    lib = N.load_scene_library()
    p = np.zeros(1, N.PILE_PARAMS_DTYPE)
    lib.bepuscene_default_pile(N.ptr(p))
    for k, v in overrides.items():
        p[k] = v
    h = ctypes.c_void_p()
    st = lib.bepuscene_make_pile(N.ptr(p), ctypes.byref(h))
    N.raise_for(st, "bepuscene_make_pile")
    return _collect(h, with_shapes=bool(p["narrow_phase"][0]))


def make_tower(body_count: int, seed: int = 1, **overrides):
    lib = N.load_scene_library()
    p = np.zeros(1, N.TOWER_PARAMS_DTYPE)
    lib.bepuscene_default_tower(N.ptr(p))
    p["body_count"] = body_count
    p["seed"] = seed
    for k, v in overrides.items():
        p[k] = v
    h = ctypes.c_void_p()
    st = lib.bepuscene_make_tower(N.ptr(p), ctypes.byref(h))
    N.raise_for(st, "bepuscene_make_tower")
    return _collect(h, with_shapes=bool(p["narrow_phase"][0]))


def make_chain(**overrides):
    """Articulated capsule chains plus loose spheres and boxes (bepuscene_make_chain)."""
    lib = N.load_scene_library()
    p = np.zeros(1, N.CHAIN_PARAMS_DTYPE)
    lib.bepuscene_default_chain(N.ptr(p))
    for k, v in overrides.items():
        p[k] = v
    h = ctypes.c_void_p()
    st = lib.bepuscene_make_chain(N.ptr(p), ctypes.byref(h))
    N.raise_for(st, "bepuscene_make_chain")
    return _collect(h)


def chains_8k(seed: int = 3):
    """The mixed contacts-and-joints workload: 8,192 chains of 16 capsules
    (radius 0.1 m, length 0.4 m, 1 kg), 45 degree limits, 20,000 loose spheres
    and boxes in a 200 x 50 x 200 m region."""
    return make_chain(seed=seed)


def _rows(q) -> np.ndarray:
    """Matrix3x3.CreateFromQuaternion (row-vector convention: world = local @ R), float64."""
    x, y, z, w = (float(v) for v in q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)],
                     [2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w)],
                     [2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)]])


def with_added_joint_types(bodies: np.ndarray, joints: np.ndarray) -> np.ndarray:
    """The joints of a chain scene re-typed in turn as ten of the added types,
    each set up from the current poses: weld, distance (the anchors' distance),
    prismatic with its linear limit, revolute velocity motor, linear servo
    motor, single-entity maximum speed, twist limit, swivel hinge, ellipse
    swing limit and point on plane.  Anchors stay the chain's."""
    j = joints.copy()
    ident = np.array([0, 0, 0, 1], np.float32)
    fmax = np.finfo(np.float32).max
    for k in range(len(j)):
        a, c = int(j["body_a"][k]), int(j["body_b"][k])
        qa = bodies["orientation"][a] if a >= 0 else ident
        qb = bodies["orientation"][c] if c >= 0 else ident
        j["orientation_a"][k], j["orientation_b"][k] = qa, qb
        j["impulse"][k] = 0
        j["flags"][k] = N.JOINT_ACTIVE
        kind = k % 10
        if kind == 0:
            j["type"][k] = N.JOINT_WELD
        elif kind == 1:
            wa = (bodies["position"][a] + j["anchor_a"][k] @ _rows(qa)) if a >= 0 else j["anchor_a"][k]
            wb = (bodies["position"][c] + j["anchor_b"][k] @ _rows(qb)) if c >= 0 else j["anchor_b"][k]
            j["type"][k] = N.JOINT_DISTANCE
            j["limit_min"][k] = float(np.linalg.norm(wb - wa))
        elif kind == 2:
            j["type"][k] = N.JOINT_PRISMATIC
            j["flags"][k] |= N.JOINT_LIMIT_ACTIVE
            j["limit_min"][k], j["limit_max"][k] = -0.01, 0.01
            j["basis_primary"][k], j["basis_x"][k], j["test_axis"][k] = (1, 0, 0), (0, 0, -1), (0, 1, 0)
        elif kind == 3:
            j["type"][k] = N.JOINT_REVOLUTE_MOTOR
            j["limit_max"][k], j["margin"][k], j["bounce_velocity_threshold"][k] = 1.0, 0.0001, fmax
            j["basis_primary"][k], j["basis_x"][k], j["test_axis"][k] = (1, 0, 0), (0, 0, -1), (0, 0, -1)
        elif kind == 4:
            j["type"][k] = N.JOINT_LINEAR_AXIS_MOTOR
            j["flags"][k] |= N.JOINT_SERVO
            j["limit_min"][k], j["margin"][k], j["bounce_velocity_threshold"][k] = 0.05, 0.0001, 50.0
            j["basis_primary"][k] = (0, 1, 0)
        elif kind == 5:
            j["type"][k] = N.JOINT_MAXIMUM_LINEAR_SPEED
            j["body_a"][k], j["body_b"][k] = (c if a < 0 else a), -1
            j["limit_min"][k], j["limit_max"][k], j["margin"][k] = 0.5, fmax, 0.00001
        elif kind == 6:
            j["type"][k] = N.JOINT_TWIST_LIMIT
            j["axis_a"][k] = j["axis_b"][k] = (1, 0, 0)
            j["constrained_1"][k], j["constrained_2"][k], j["basis_x"][k] = (0, 0, -1), (0, 1, 0), (0, 0, -1)
            j["limit_min"][k], j["limit_max"][k] = -0.5, 0.5
        elif kind == 7:
            j["type"][k] = N.JOINT_SWIVEL_HINGE
            j["axis_a"][k], j["axis_b"][k] = (1, 0, 0), (0, 1, 0)
        elif kind == 8:
            j["type"][k] = N.JOINT_ELLIPSE_SWING_LIMIT
            j["axis_a"][k], j["constrained_1"][k], j["constrained_2"][k] = (0, 1, 0), (1, 0, 0), (0, 0, 1)
            j["axis_b"][k] = (0, 1, 0)
            j["limit_min"][k], j["limit_max"][k] = 0.5, 0.3
        else:
            j["type"][k] = N.JOINT_POINT_ON_PLANE
            j["axis_a"][k] = (0, 1, 0)
    return j


def pile_1k(seed: int = 1234):
    return make_pile(seed=seed)


def pile_64k(seed: int = 1234, nx: int = 64, ny: int = 16, nz: int = 64):
    return make_pile(nx=nx, ny=ny, nz=nz, spacing=2.0, size_min=0.5, size_max=1.5, density=1.0, jitter=0.1,
                     friction_min=0.4, friction_max=0.8, ground_size=(140.0, 1.0, 140.0), seed=seed)


def dropped_pile(seed: int = 1234, nx: int = 64, ny: int = 16, nz: int = 64, drop_spacing: float = 2.0):
    """pile_64k's boxes (sizes U(0.5, 1.5) per axis, density 1, friction
    U(0.4, 0.8), horizontal jitter +-0.1) on a grid with drop_spacing between
    layers too, at rest in the air above the static ground and without
    manifolds: the pile before it settles.  Returns (bodies, shapes, per-body
    friction)."""
    lib = N.load_scene_library()
    p = np.zeros(1, N.PILE_PARAMS_DTYPE)
    lib.bepuscene_default_pile(N.ptr(p))
    for k, v in dict(nx=nx, ny=ny, nz=nz, spacing=2.0, size_min=0.5, size_max=1.5, density=1.0, jitter=0.1,
                     friction_min=0.4, friction_max=0.8, ground_size=(140.0, 1.0, 140.0), seed=seed,
                     narrow_phase=1, drop_spacing=drop_spacing).items():
        p[k] = v
    h = ctypes.c_void_p()
    st = lib.bepuscene_make_pile(N.ptr(p), ctypes.byref(h))
    N.raise_for(st, "bepuscene_make_pile")
    return _collect(h, with_friction=True)


def pile_64k_collide(seed: int = 1234, nx: int = 64, ny: int = 16, nz: int = 64):
    """pile_64k with the narrow phase on the device: the same boxes, every pair
    within the contact distance an empty GENERATED manifold; returns
    (bodies, manifolds, joints, shapes)."""
    return make_pile(nx=nx, ny=ny, nz=nz, spacing=2.0, size_min=0.5, size_max=1.5, density=1.0, jitter=0.1,
                     friction_min=0.4, friction_max=0.8, ground_size=(140.0, 1.0, 140.0), seed=seed,
                     narrow_phase=1)


def batch_body_counts(n: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """Scene sizes log-uniform in [lo, hi] (the batching and serving workloads)."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n)).round().astype(np.int64)


def tower_batch(n: int = 4096, lo: int = 8, hi: int = 2048, seed: int = 4):
    """n independent tower scenes, body counts log-uniform in [lo, hi]."""
    return [make_tower(int(k), seed=seed * 100003 + i) for i, k in enumerate(batch_body_counts(n, lo, hi, seed))]


def contact_count(manifolds: np.ndarray) -> int:
    return int(manifolds["contact_count"].sum())
