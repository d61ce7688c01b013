"""Joint records for the parity tests: chain joints re-typed as the added
joint types, with each type's fields set up from the bodies' current poses,
and group records given continuation children."""
import numpy as np

from bepuphysics1_gb300 import native as N

NEW_TYPES = (N.JOINT_WELD, N.JOINT_NO_ROTATION, N.JOINT_DISTANCE, N.JOINT_DISTANCE_LIMIT, N.JOINT_POINT_ON_PLANE,
             N.JOINT_TWIST, N.JOINT_POINT_ON_LINE, N.JOINT_PRISMATIC, N.JOINT_LINE_SLIDER, N.JOINT_UNIVERSAL,
             N.JOINT_TWIST_LIMIT, N.JOINT_LINEAR_AXIS_LIMIT, N.JOINT_ELLIPSE_SWING_LIMIT,
             N.JOINT_SWIVEL_HINGE_ANGULAR, N.JOINT_SWIVEL_HINGE, N.JOINT_REVOLUTE_MOTOR, N.JOINT_TWIST_MOTOR,
             N.JOINT_LINEAR_AXIS_MOTOR)
MOTORS = (N.JOINT_REVOLUTE_MOTOR, N.JOINT_TWIST_MOTOR, N.JOINT_LINEAR_AXIS_MOTOR)
SPEED_LIMITS = (N.JOINT_MAXIMUM_LINEAR_SPEED, N.JOINT_MAXIMUM_ANGULAR_SPEED)
NEW_TYPES = NEW_TYPES + SPEED_LIMITS + (N.JOINT_PLANE_SLIDER, N.JOINT_ANGULAR_MOTOR,
                                       N.JOINT_SINGLE_ENTITY_ANGULAR_MOTOR, N.JOINT_SINGLE_ENTITY_LINEAR_MOTOR)


def _unit(v):
    return v / np.linalg.norm(v)


def _perpendicular_pair(d):
    """PointOnLineJoint.UpdateRestrictedAxes (PointOnLineJoint.cs:465-474) in float64."""
    r1 = np.cross((0, 1, 0), d)
    if r1 @ r1 < .001:
        r1 = np.cross((1, 0, 0), d)
    r2 = np.cross(d, r1)
    return _unit(r1), _unit(r2)


def _rows(q):
    x, y, z, w = (float(v) for v in q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)],
                     [2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w)],
                     [2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)]])


def convert(b, j, types, seed):
    """The chain joints re-typed: welds and no-rotation joints keep the pose
    they are made in (the constructors' initial orientations), distance joints
    keep the anchors' current distance, distance limits bracket it."""
    j = j.copy()
    rng = np.random.default_rng(seed)
    ident = np.array([0, 0, 0, 1], np.float32)
    for k in range(len(j)):
        t = types[rng.integers(len(types))]
        a, bb = int(j["body_a"][k]), int(j["body_b"][k])
        qa = b["orientation"][a] if a >= 0 else ident
        qb = b["orientation"][bb] if bb >= 0 else ident
        wa = (b["position"][a] + j["anchor_a"][k] @ _rows(qa)) if a >= 0 else j["anchor_a"][k]
        wb = (b["position"][bb] + j["anchor_b"][k] @ _rows(qb)) if bb >= 0 else j["anchor_b"][k]
        d = float(np.linalg.norm(wb - wa))
        j["type"][k] = t
        j["impulse"][k] = 0
        j["orientation_a"][k] = qa
        j["orientation_b"][k] = qb
        if t == N.JOINT_DISTANCE:
            j["limit_min"][k] = d * rng.uniform(0.95, 1.05)
        elif t == N.JOINT_DISTANCE_LIMIT:
            lo = d * rng.uniform(0.7, 1.02)
            j["limit_min"][k], j["limit_max"][k] = lo, lo + d * rng.uniform(0.0, 0.2)
            j["bounciness"][k] = rng.choice([0.0, 0.5])
        elif t in (N.JOINT_POINT_ON_PLANE, N.JOINT_PLANE_SLIDER):
            n = rng.normal(size=3)
            j["axis_a"][k] = n / np.linalg.norm(n)
        elif t in (N.JOINT_POINT_ON_LINE, N.JOINT_PRISMATIC, N.JOINT_LINE_SLIDER):
            ra, rb = _rows(qa), _rows(qb)
            d = _unit(rng.normal(size=3))  # the line direction in A's frame
            r1, r2 = _perpendicular_pair(d)
            j["basis_primary"][k], j["basis_x"][k], j["test_axis"][k] = d, r1, r2
            if t == N.JOINT_LINE_SLIDER:  # RevoluteAngularJoint about the line
                wd = d @ ra
                c1, c2 = _perpendicular_pair(wd)
                j["axis_a"][k], j["axis_b"][k] = d, wd @ rb.T
                j["constrained_1"][k], j["constrained_2"][k] = c1 @ ra.T, c2 @ ra.T
        if t in (N.JOINT_LINEAR_AXIS_LIMIT, N.JOINT_PRISMATIC, N.JOINT_LINE_SLIDER):
            # limits around the anchors' separation along the axis (zero for chain links)
            if t == N.JOINT_LINEAR_AXIS_LIMIT:
                j["basis_primary"][k] = _unit(rng.normal(size=3))
            lo = rng.uniform(-0.03, 0.005)
            j["limit_min"][k], j["limit_max"][k] = lo, lo + rng.uniform(0.0, 0.03)
            j["bounciness"][k] = rng.choice([0.0, 0.5])
            if t != N.JOINT_LINEAR_AXIS_LIMIT and rng.random() < 0.6:
                j["flags"][k] |= N.JOINT_LIMIT_ACTIVE
        if t == N.JOINT_TWIST_LIMIT:
            # TwistLimit.SetupJointTransforms (TwistLimit.cs:165-197) for a shared world axis
            ax = _unit(rng.normal(size=3))
            ra, rb = _rows(qa), _rows(qb)
            x = np.cross(ax, (0, 1, 0))
            if x @ x < 1e-7:
                x = np.cross(ax, (1, 0, 0))
            x = _unit(x)
            y = _unit(np.cross(ax, x))
            j["axis_a"][k], j["constrained_1"][k], j["constrained_2"][k] = ax @ ra.T, x @ ra.T, y @ ra.T
            j["axis_b"][k], j["basis_x"][k] = ax @ rb.T, x @ rb.T
            lo = rng.uniform(-0.3, 0.02)
            j["limit_min"][k], j["limit_max"][k] = lo, lo + rng.uniform(0.0, 0.3)
            j["bounciness"][k] = rng.choice([0.0, 0.5])
        if t == N.JOINT_ELLIPSE_SWING_LIMIT:
            # EllipseSwingLimit.SetupJointTransforms (EllipseSwingLimit.cs:138-160)
            ax = _unit(rng.normal(size=3))
            ra, rb = _rows(qa), _rows(qb)
            x = np.cross(ax, (0, 1, 0))
            if x @ x < 1e-7:
                x = np.cross(ax, (1, 0, 0))
            y = np.cross(ax, x)
            j["axis_a"][k], j["constrained_1"][k], j["constrained_2"][k] = ax @ ra.T, _unit(x) @ ra.T, _unit(y) @ ra.T
            # B's twist axis tilted off A's primary by up to 0.3 rad: some limits start violated
            tilt = _unit(np.cross(ax, rng.normal(size=3)))
            ang = rng.uniform(0.0, 0.3)
            j["axis_b"][k] = _unit(ax * np.cos(ang) + tilt * np.sin(ang)) @ rb.T
            j["limit_min"][k], j["limit_max"][k] = rng.uniform(0.005, 0.2), rng.uniform(0.005, 0.2)
            j["bounciness"][k] = rng.choice([0.0, 0.5])
        if t == N.JOINT_SINGLE_ENTITY_ANGULAR_MOTOR:  # on the link, the world as body B
            if a < 0:
                a, qa = bb, qb
            j["body_a"][k], j["body_b"][k] = a, -1
        if t == N.JOINT_SINGLE_ENTITY_LINEAR_MOTOR:  # the link's anchor point towards a nearby goal
            if a < 0:
                a, qa = bb, qb
                j["anchor_a"][k] = j["anchor_b"][k]
            j["body_a"][k], j["body_b"][k] = a, -1
            servo = rng.random() < 0.5
            j["flags"][k] |= N.JOINT_SERVO if servo else 0
            wp = b["position"][a] + j["anchor_a"][k] @ _rows(qa)
            j["anchor_b"][k] = wp + rng.uniform(-0.05, 0.05, 3) * (rng.random() < 0.8)
            j["axis_a"][k] = rng.uniform(-0.5, 0.5, 3)
            j["margin"][k] = 0.0001
            j["bounciness"][k] = rng.choice([0.0, 0.3])
            j["bounce_velocity_threshold"][k] = rng.choice([np.finfo(np.float32).max, 5.0])
            j["max_corrective_velocity"][k] = rng.choice([np.finfo(np.float32).max, 1.0])
        if t in (N.JOINT_ANGULAR_MOTOR, N.JOINT_SINGLE_ENTITY_ANGULAR_MOTOR):
            ra = _rows(qa)
            ax = _unit(rng.normal(size=3))
            x = _unit(np.cross(ax, rng.normal(size=3)))
            y = np.cross(ax, x)
            j["axis_a"][k], j["constrained_1"][k], j["constrained_2"][k] = ax @ ra.T, x @ ra.T, y @ ra.T
            servo = rng.random() < 0.5
            j["flags"][k] |= N.JOINT_SERVO if servo else 0
            g = _unit(rng.normal(size=4))
            j["orientation_a"][k] = g if g[3] >= 0 else -g
            j["anchor_a"][k] = rng.uniform(-1, 1, 3)
            j["margin"][k] = 0.0001
            j["bounciness"][k] = rng.choice([0.0, 0.3])
            j["bounce_velocity_threshold"][k] = rng.choice([np.finfo(np.float32).max, 5.0])
            j["max_corrective_velocity"][k] = rng.choice([np.finfo(np.float32).max, 2.0])
        if t in SPEED_LIMITS:  # single-entity: on the link, the world as body B
            j["body_a"][k], j["body_b"][k] = (bb if a < 0 else a), -1
            j["limit_min"][k] = rng.uniform(0.0, 0.2) if t == N.JOINT_MAXIMUM_LINEAR_SPEED else rng.uniform(0.0, 0.5)
            j["limit_max"][k] = rng.choice([np.finfo(np.float32).max, 2.0])
            j["margin"][k] = 0.00001
        if t in MOTORS:
            servo = rng.random() < 0.5
            j["flags"][k] |= N.JOINT_SERVO if servo else 0
            linear = t == N.JOINT_LINEAR_AXIS_MOTOR
            j["limit_min"][k] = rng.uniform(-0.05, 0.05) if linear else rng.uniform(-np.pi, np.pi)
            j["limit_max"][k] = rng.uniform(-1.0, 1.0)
            j["margin"][k] = 0.0001
            j["bounciness"][k] = rng.choice([0.0, 0.3])
            j["bounce_velocity_threshold"][k] = rng.choice([np.finfo(np.float32).max, 5.0])
            ra, rb = _rows(qa), _rows(qb)
            ax = _unit(rng.normal(size=3))
            if t == N.JOINT_REVOLUTE_MOTOR:
                x = _unit(np.cross(ax, rng.normal(size=3)))
                ang = rng.uniform(-np.pi, np.pi)
                xt = x * np.cos(ang) + np.cross(ax, x) * np.sin(ang)
                j["basis_primary"][k], j["basis_x"][k], j["test_axis"][k] = ax @ ra.T, x @ ra.T, xt @ rb.T
            elif t == N.JOINT_TWIST_MOTOR:
                x = _unit(np.cross(ax, rng.normal(size=3)))
                y = _unit(np.cross(ax, x))
                j["axis_a"][k], j["constrained_1"][k], j["constrained_2"][k] = ax @ ra.T, x @ ra.T, y @ ra.T
                j["axis_b"][k], j["basis_x"][k] = ax @ rb.T, x @ rb.T
            else:
                j["basis_primary"][k] = ax @ ra.T
        if t in (N.JOINT_SWIVEL_HINGE_ANGULAR, N.JOINT_SWIVEL_HINGE):
            # a hinge axis on A and a twist axis on B, perpendicular up to 0.1 rad
            ra, rb = _rows(qa), _rows(qb)
            h = _unit(rng.normal(size=3))
            t0 = _unit(np.cross(h, rng.normal(size=3)))
            e = rng.uniform(-0.1, 0.1)
            j["axis_a"][k], j["axis_b"][k] = h @ ra.T, _unit(t0 * np.cos(e) + h * np.sin(e)) @ rb.T
        if t in (N.JOINT_TWIST, N.JOINT_UNIVERSAL):
            # TwistJoint.Initialize (TwistJoint.cs:340-365) for a shared world axis
            ax = rng.normal(size=3)
            ax /= np.linalg.norm(ax)
            ra, rb = _rows(qa), _rows(qb)
            y = np.cross(ax, (0, 1, 0))
            if y @ y < 1e-7:
                y = np.cross(ax, (1, 0, 0))
            y /= np.linalg.norm(y)
            la = ax @ ra.T
            j["axis_a"][k] = la
            j["axis_b"][k] = ax @ rb.T
            j["constrained_1"][k] = y @ ra.T
            j["constrained_2"][k] = np.cross(la, y @ ra.T)
            j["basis_x"][k] = y @ rb.T
    return j


# The children a group record may take as continuation records, in the order
# the group's constructor Adds them (RevoluteJoint.cs:88-91,
# PrismaticJoint.cs:57-60, LineSliderJoint.cs:55-58, UniversalJoint.cs:54-57,
# SwivelHingeJoint.cs:96-101, PlaneSliderJoint.cs:64-68).
GROUP_CHILDREN = {
    N.JOINT_REVOLUTE: (N.JOINT_REVOLUTE_MOTOR,),
    N.JOINT_PRISMATIC: (N.JOINT_LINEAR_AXIS_MOTOR,),
    N.JOINT_LINE_SLIDER: (N.JOINT_LINEAR_AXIS_MOTOR,),
    N.JOINT_UNIVERSAL: (N.JOINT_TWIST_LIMIT, N.JOINT_TWIST_MOTOR),
    N.JOINT_SWIVEL_HINGE: (N.JOINT_REVOLUTE_LIMIT, N.JOINT_REVOLUTE_MOTOR, N.JOINT_TWIST_LIMIT,
                           N.JOINT_TWIST_MOTOR),
    N.JOINT_PLANE_SLIDER: (N.JOINT_LINEAR_AXIS_LIMIT, N.JOINT_LINEAR_AXIS_MOTOR, N.JOINT_LINEAR_AXIS_LIMIT,
                           N.JOINT_LINEAR_AXIS_MOTOR),
}


def _revolute_limit(b, rec, rng):
    """RevoluteLimit fields for the record's bodies: a random basis on A, a test
    axis on B at a random angle about the primary axis, limits that some of
    the angles violate."""
    ident = np.array([0, 0, 0, 1], np.float32)
    a, c = int(rec["body_a"][0]), int(rec["body_b"][0])
    ra = _rows(b["orientation"][a] if a >= 0 else ident)
    rb = _rows(b["orientation"][c] if c >= 0 else ident)
    ax = _unit(rng.normal(size=3))
    x = _unit(np.cross(ax, rng.normal(size=3)))
    ang = rng.uniform(-np.pi, np.pi)
    xt = x * np.cos(ang) + np.cross(ax, x) * np.sin(ang)
    rec["basis_primary"][0], rec["basis_x"][0], rec["test_axis"][0] = ax @ ra.T, x @ ra.T, xt @ rb.T
    lo = rng.uniform(-np.pi / 2, 0.2)
    rec["limit_min"][0], rec["limit_max"][0] = lo, lo + rng.uniform(0.0, 1.5)
    rec["margin"][0] = rng.choice([0.0, 0.005])
    rec["bounciness"][0] = rng.choice([0.0, 0.5])


def with_group_children(b, j, seed, heads=tuple(GROUP_CHILDREN), keep=0.75, inactive_children=0.0,
                        inactive_groups=0.0):
    """The chain's revolute joints re-typed as group records (heads) followed
    by continuation records of the children each takes, every child kept with
    probability `keep` (the first child always).  `inactive_children` of the
    children and `inactive_groups` of the groups are left inactive.  Other
    joints stay as they are."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(len(j)):
        rec = j[k:k + 1].copy()
        if int(rec["type"][0]) != N.JOINT_REVOLUTE:
            out.append(rec)
            continue
        t = heads[rng.integers(len(heads))]
        head = rec if t == N.JOINT_REVOLUTE else convert(b, rec, (t,), int(rng.integers(1 << 30)))
        head["impulse"][0] = 0
        if rng.random() < inactive_groups:
            head["flags"][0] &= ~np.uint32(N.JOINT_ACTIVE)
        out.append(head)
        for n, ct in enumerate(GROUP_CHILDREN[t]):
            if n and rng.random() >= keep:
                continue
            child = convert(b, j[k:k + 1].copy(), (ct,), int(rng.integers(1 << 30)))
            if ct == N.JOINT_REVOLUTE_LIMIT:
                _revolute_limit(b, child, rng)
            servo = np.uint32(child["flags"][0]) & np.uint32(N.JOINT_SERVO)
            active = np.uint32(0 if rng.random() < inactive_children else N.JOINT_ACTIVE)
            child["flags"][0] = servo | active | np.uint32(N.JOINT_GROUP_CONTINUATION)
            child["body_a"][0], child["body_b"][0] = head["body_a"][0], head["body_b"][0]
            child["impulse"][0] = 0
            out.append(child)
    return np.concatenate(out) if out else j.copy()


def as_separate_children(j):
    """The same records with every continuation made a joint of its own: active
    when it and its group are."""
    s = j.copy()
    group_active = True
    for k in range(len(s)):
        f = int(s["flags"][k])
        if f & N.JOINT_GROUP_CONTINUATION:
            keep = (f & ~(N.JOINT_GROUP_CONTINUATION | N.JOINT_ACTIVE)) | \
                (N.JOINT_ACTIVE if (f & N.JOINT_ACTIVE) and group_active else 0)
            s["flags"][k] = keep
        else:
            group_active = bool(f & N.JOINT_ACTIVE)
    return s
