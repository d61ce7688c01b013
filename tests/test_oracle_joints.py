"""Known-answer tests pinning the oracle's joint restatements.

The reference ships no solver golden vectors, so each joint is pinned by a
hand-derived closed form of one prestep and one solve iteration from rest
(no gravity, no damping, no warm start), evaluated here in float64:
  BallSocketJoint.Update/SolveIteration   BallSocketJoint.cs:210-278, 318-372
  SwingLimit.Update/SolveIteration        SwingLimit.cs:211-331
  RevoluteLimit.Update                    RevoluteLimit.cs:285-575
and the switches the reference makes between active and inactive limits.
"""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300.solver import default_settings

DT = np.float32(1 / 60)
K, D = 600000.0, 90000.0  # SpringSettings defaults


def _settings(iterations=1):
    s = default_settings()
    s["gravity"] = (0, 0, 0)
    s["iteration_limit"] = iterations
    return s


def _body(pos, inv_mass=1.0, inv_inertia=(2.0, 3.0, 4.0), quat=(0, 0, 0, 1)):
    b = np.zeros(1, N.BODY_DTYPE)
    b["position"] = pos
    b["orientation"] = quat
    b["inverse_mass"] = inv_mass
    b["local_inverse_inertia"] = np.diag(inv_inertia).reshape(9)
    b["is_dynamic"] = 1
    return b


def _joint(jtype, a, b):
    j = np.zeros(1, N.JOINT_DTYPE)
    j["type"], j["body_a"], j["body_b"], j["flags"] = jtype, a, b, N.JOINT_ACTIVE
    j["margin"], j["bounce_velocity_threshold"] = 0.005, 1.0
    j["max_corrective_velocity"] = np.finfo(np.float32).max
    j["spring_stiffness"], j["spring_damping"] = K, D
    return j


def _spring(dt):
    m = 1 / (dt * K + D)
    return K * m, (1 / dt) * m  # error reduction, softness


def _cross_matrix(v):
    return np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])


def _step(bodies, joints):
    o = oracle.OracleSpace(_settings(), bodies, np.zeros(0, N.MANIFOLD_DTYPE), joints)
    o.set_order_mode(oracle.ORDER_IDENTITY)
    o.step(DT, N.STEP_SOLVE, 1)
    return o.get_bodies(), o.get_constraints()[1]


def _rot_z(phi):
    return (0.0, 0.0, np.sin(phi / 2), np.cos(phi / 2))


def test_ball_socket_to_world_closed_form():
    # body B at (0, -1, 0) hangs from the world anchor at the origin by a local
    # anchor 1.1 above its centre: position error (0, 0.1, 0)
    b = _body((0, -1, 0))
    j = _joint(N.JOINT_BALL_SOCKET, -1, 0)
    j["anchor_a"] = (0, 0, 0)
    j["anchor_b"] = (0, 1.1, 0)
    ob, oj = _step(b, j)
    dt = float(DT)
    erp, soft = _spring(dt)
    r = np.array([0, 1.1, 0])
    inv_i = np.diag([2.0, 3.0, 4.0])
    rx = _cross_matrix(r)
    k = np.eye(3) * 1.0 - rx @ inv_i @ rx + soft * np.eye(3)
    # Matrix3x3 is row-vector: lambda = v * M with M = K^-1 (K is symmetric here)
    err = np.array([0, -1, 0]) + r
    bias = -erp * err
    lam = bias @ np.linalg.inv(k)
    v = lam * 1.0
    w = np.cross(r, lam) @ inv_i
    np.testing.assert_allclose(oj["impulse"][0, :3], lam, rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(ob["linear_velocity"][0], v, rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(ob["angular_velocity"][0], w, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("phi_deg,active", [(30.0, False), (60.0, True)])
def test_swing_limit_switch(phi_deg, active):
    phi = np.radians(phi_deg)
    b = _body((0, 0, 0), quat=_rot_z(phi))
    j = _joint(N.JOINT_SWING_LIMIT, -1, 0)
    j["axis_a"] = (0, 1, 0)
    j["axis_b"] = (0, 1, 0)
    j["limit_min"] = np.float32(np.cos(np.radians(45.0)))
    j["impulse"][0, 0] = 0.25  # a stale impulse: zeroed when the limit is not reached (SwingLimit.cs:259-266)
    ob, oj = _step(b, j)
    if not active:
        assert oj["impulse"][0, 0] == 0.0
        assert np.all(ob["angular_velocity"][0] == 0.0)
        return
    dt = float(DT)
    erp, soft = _spring(dt)
    axis_a = np.array([0, 1.0, 0])
    axis_b = np.array([-np.sin(phi), np.cos(phi), 0])
    hinge = np.cross(axis_a, axis_b)
    # the body inertia in world: R^T L R for a rotation about z
    c, s = np.cos(phi), np.sin(phi)
    rot = np.array([[c, s, 0], [-s, c, 0], [0, 0, 1]])  # CreateFromQuaternion, row-vector convention
    inv_i = rot.T @ np.diag([2.0, 3.0, 4.0]) @ rot
    error = max(0.0, np.cos(np.radians(45.0)) - np.dot(axis_a, axis_b) - 0.005)
    bias = erp * error
    v2i = 1 / (soft + hinge @ inv_i @ hinge)
    # warm start applies the stale 0.25 first; one solve from that state
    w_warm = -(hinge * 0.25) @ inv_i
    lam = (-(np.zeros(3) - w_warm) @ hinge + bias - soft * 0.25) * v2i
    acc = max(0.25 + lam, 0.0)
    w = w_warm - (hinge * (acc - 0.25)) @ inv_i
    np.testing.assert_allclose(oj["impulse"][0, 0], acc, rtol=1e-5)
    np.testing.assert_allclose(ob["angular_velocity"][0], w, rtol=1e-4, atol=1e-7)


@pytest.mark.parametrize("phi_deg,active", [(20.0, False), (-20.0, False), (60.0, True), (-60.0, True)])
def test_revolute_limit_planes(phi_deg, active):
    # free axis z; A = world with x axis (1,0,0); B rotated about z by phi with
    # local test axis x: the test axis makes angle phi with the basis x axis
    phi = np.radians(phi_deg)
    b = _body((0, 0, 0), quat=_rot_z(phi))
    j = _joint(N.JOINT_REVOLUTE_LIMIT, -1, 0)
    j["basis_primary"] = (0, 0, 1)
    j["basis_x"] = (1, 0, 0)
    j["test_axis"] = (1, 0, 0)
    j["limit_min"] = np.float32(-np.pi / 4)
    j["limit_max"] = np.float32(np.pi / 4)
    j["impulse"][0, :2] = (0.5, 0.5)
    ob, oj = _step(b, j)
    imp = oj["impulse"][0, :2]
    if not active:
        assert np.all(imp == 0.0)
        assert np.all(ob["angular_velocity"][0] == 0.0)
        return
    # exactly one plane is violated; the other impulse is zeroed (RevoluteLimit.cs:365-395)
    assert (imp[0] == 0.0) != (imp[1] == 0.0)
    # the correction turns B back toward the allowed range about the free axis
    wz = ob["angular_velocity"][0][2]
    assert np.sign(wz) == -np.sign(phi)


def test_no_rotation_to_world_closed_form():
    """NoRotationJoint.Update / SolveIteration (NoRotationJoint.cs:160-243):
    body B turned by phi about z against the world; one solve from rest turns
    it back about z with lambda = erp * phi / (I_zz + softness)."""
    phi = np.radians(10.0)
    b = _body((0, 0, 0), quat=_rot_z(phi))
    j = _joint(N.JOINT_NO_ROTATION, -1, 0)
    j["orientation_a"] = (0, 0, 0, 1)
    j["orientation_b"] = (0, 0, 0, 1)
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    # error = axis * angle of conj(qB): (0, 0, -phi); bias = -erp * error
    lam_z = erp * phi / (4.0 + soft)
    np.testing.assert_allclose(oj["impulse"][0, :3], (0, 0, lam_z), rtol=1e-4, atol=1e-9)
    # B takes the negated impulse: w = -lambda * I_zz
    np.testing.assert_allclose(ob["angular_velocity"][0], (0, 0, -4.0 * lam_z), rtol=1e-4, atol=1e-8)


def test_distance_joint_to_world_closed_form():
    """DistanceJoint (DistanceJoint.cs:226-352): B 0.1 beyond its distance of 2
    from a world anchor is pulled back along the line, no angular part."""
    b = _body((2.1, 0, 0))
    j = _joint(N.JOINT_DISTANCE, -1, 0)
    j["limit_min"] = 2.0
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    vti = 1 / (soft + 1.0)
    lam = (-0.1 * erp) * vti  # error = distance - current
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-5)
    np.testing.assert_allclose(ob["linear_velocity"][0], (lam, 0, 0), rtol=1e-5, atol=1e-9)
    assert np.all(ob["angular_velocity"][0] == 0)


@pytest.mark.parametrize("x,active", [(1.5, False), (2.3, True), (0.7, True)])
def test_distance_limit_switch(x, active):
    """DistanceLimit (DistanceLimit.cs:260-430): inside [1, 2] nothing acts and
    a stale impulse is cleared; beyond either end a non-negative impulse
    pushes back by the error less the margin."""
    b = _body((x, 0, 0))
    j = _joint(N.JOINT_DISTANCE_LIMIT, -1, 0)
    j["limit_min"], j["limit_max"] = 1.0, 2.0
    j["impulse"][0, 0] = 0.0 if active else 0.3
    ob, oj = _step(b, j)
    if not active:
        assert oj["impulse"][0, 0] == 0 and np.all(ob["linear_velocity"][0] == 0)
        return
    erp, soft = _spring(float(DT))
    error = (x - 2.0 - 0.005) if x > 2 else (1.0 - 0.005 - x)
    lam = erp * error / (soft + 1.0)
    assert oj["impulse"][0, 0] > 0
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(abs(ob["linear_velocity"][0, 0]), lam, rtol=1e-4)
    assert np.sign(ob["linear_velocity"][0, 0]) == (-1 if x > 2 else 1)


def test_weld_is_ball_socket_then_no_rotation():
    """WeldJoint (WeldJoint.cs:15-55) solves its ball socket, then its
    no-rotation joint, as one SolverGroup: the impulses land in [0..2] and
    [3..5], each one nonzero for an offset and turned body."""
    b = _body((0.05, -1, 0), quat=_rot_z(np.radians(5.0)))
    j = _joint(N.JOINT_WELD, -1, 0)
    j["anchor_b"] = (0, 1, 0)
    j["orientation_a"] = (0, 0, 0, 1)
    j["orientation_b"] = (0, 0, 0, 1)
    _, oj = _step(b, j)
    assert np.abs(oj["impulse"][0, :3]).max() > 0 and np.abs(oj["impulse"][0, 3:6]).max() > 0
    assert np.all(oj["impulse"][0, 6:] == 0)


def test_point_on_plane_to_world_closed_form():
    """PointOnPlaneJoint (PointOnPlaneJoint.cs:212-306): B's centre 0.1 above the
    world's y = 0 plane is pushed down; the solve returns the signed lambda."""
    b = _body((0.3, 0.1, -0.2))
    j = _joint(N.JOINT_POINT_ON_PLANE, -1, 0)
    j["axis_a"] = (0, 1, 0)
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    lam = (erp * 0.1) / (1.0 + soft)  # negative effective mass times the bias
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(ob["linear_velocity"][0], (0, -lam, 0), rtol=1e-4, atol=1e-9)


def test_twist_to_world_closed_form():
    """TwistJoint (TwistJoint.cs:204-300): B twisted by phi about the shared x
    axis; the error is atan2 of the measured y axis, the jacobian x."""
    phi = np.radians(12.0)
    b = _body((0, 0, 0), quat=(np.sin(phi / 2), 0, 0, np.cos(phi / 2)))
    j = _joint(N.JOINT_TWIST, -1, 0)
    j["axis_a"] = j["axis_b"] = (1, 0, 0)
    j["constrained_1"] = (0, 0, -1)  # A's local y: cross(x, up) normalised
    j["constrained_2"] = (0, 1, 0)   # A's local z: cross(axis, y)
    j["basis_x"] = (0, 0, -1)        # B's local y
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    # B's y axis turned by phi about x, measured in A's (y, z) frame: error = phi
    lam = (-phi * erp) / (soft + 2.0)  # I_xx = 2, jacobianB = x
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(ob["angular_velocity"][0], (2.0 * lam, 0, 0), rtol=1e-4, atol=1e-8)


def test_point_on_line_to_world_closed_form():
    """PointOnLineJoint (PointOnLineJoint.cs:247-438): B's centre 0.1 off the
    world's x axis is pulled back along the restricted axis (0, 1, 0)."""
    b = _body((0.5, 0.1, 0))
    j = _joint(N.JOINT_POINT_ON_LINE, -1, 0)
    j["basis_primary"] = (1, 0, 0)  # line direction
    j["basis_x"] = (0, 0, -1)       # restricted axes of UpdateRestrictedAxes for x
    j["test_axis"] = (0, 1, 0)
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    y = erp * 0.1 / (1.0 + soft)
    np.testing.assert_allclose(oj["impulse"][0, :2], (0, y), rtol=1e-4, atol=1e-9)
    np.testing.assert_allclose(ob["linear_velocity"][0], (0, -y, 0), rtol=1e-4, atol=1e-9)


def _twist_limit_z(phi, lo, hi, error=0.0):
    """B turned by phi about the world z axis, a twist limit about z to the world."""
    b = _body((0, 0, 0), quat=_rot_z(phi))
    j = _joint(N.JOINT_TWIST_LIMIT, -1, 0)
    j["axis_a"] = j["axis_b"] = (0, 0, 1)   # basis primaries
    j["constrained_1"] = (1, 0, 0)           # basis A x
    j["constrained_2"] = (0, 1, 0)           # basis A y
    j["basis_x"] = (1, 0, 0)                 # basis B x
    j["limit_min"], j["limit_max"] = lo, hi
    j["impulse"][0, 1] = error
    return b, j


@pytest.mark.parametrize("phi", [0.1, -0.15])
def test_twist_limit_inside_clears_impulse_and_error(phi):
    """TwistLimit (TwistLimit.cs:238-260): an angle inside [min, max] turns the
    limit off and zeroes its impulse and its error."""
    b, j = _twist_limit_z(phi, -0.2, 0.2, error=0.3)
    j["impulse"][0, 0] = 0.4
    ob, oj = _step(b, j)
    assert oj["impulse"][0, 0] == 0 and oj["impulse"][0, 1] == 0
    assert np.all(ob["angular_velocity"][0] == 0)


def test_twist_limit_beyond_maximum_closed_form():
    """Past the maximum by 0.3 rad: error -0.3 (TwistLimit.cs:334-339), the
    jacobian A = z (the previous error was 0), B pushed back about -z."""
    b, j = _twist_limit_z(0.5, -0.2, 0.2)
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    lam = (0.3 - 0.005) * erp / (soft + 4.0)  # I_zz = 4, jacobianB = -z
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(oj["impulse"][0, 1], -0.3, rtol=1e-4)
    np.testing.assert_allclose(ob["angular_velocity"][0], (0, 0, -4.0 * lam), rtol=1e-4, atol=1e-8)


def test_twist_limit_jacobian_follows_previous_error():
    """Past the minimum the error is positive (+0.3), but the jacobian of that
    step still follows the previous error (0): B is pushed further about -z.
    With the error +0.3 kept, the next step's jacobian flips and B is pushed
    back about +z (TwistLimit.cs:284-312)."""
    erp, soft = _spring(float(DT))
    lam = (0.3 - 0.005) * erp / (soft + 4.0)
    b, j = _twist_limit_z(-0.5, -0.2, 0.2, error=0.0)
    ob, oj = _step(b, j)
    np.testing.assert_allclose(oj["impulse"][0, 1], 0.3, rtol=1e-4)
    np.testing.assert_allclose(ob["angular_velocity"][0], (0, 0, -4.0 * lam), rtol=1e-4, atol=1e-8)
    b, j = _twist_limit_z(-0.5, -0.2, 0.2, error=0.3)
    ob, oj = _step(b, j)
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(ob["angular_velocity"][0], (0, 0, 4.0 * lam), rtol=1e-4, atol=1e-8)


def test_twist_limit_angle_setters_wrap_the_minimum():
    """MinimumAngle wraps into (-pi, pi]; MaximumAngle is only reduced modulo
    2 pi (TwistLimit.cs:50-75): a minimum of 2 pi - 0.2 acts as -0.2."""
    b, j = _twist_limit_z(0.5, 2 * np.pi - 0.2, 0.2)
    ob, oj = _step(b, j)
    b2, j2 = _twist_limit_z(0.5, -0.2, 0.2)
    ob2, oj2 = _step(b2, j2)
    np.testing.assert_allclose(oj["impulse"][0, :2], oj2["impulse"][0, :2], rtol=1e-5)


@pytest.mark.parametrize("x,side", [(0.5, 0), (1.5, 1), (-0.4, -1)])
def test_linear_axis_limit_closed_form(x, side):
    """LinearAxisLimit (LinearAxisLimit.cs:290-447): B's centre at x along the
    world's x axis with limits [0, 1].  Inside nothing acts and a stale impulse
    is cleared; above the maximum the impulse is non-negative, below the
    minimum non-positive, and B is pushed back either way."""
    b = _body((x, 0, 0))
    j = _joint(N.JOINT_LINEAR_AXIS_LIMIT, -1, 0)
    j["basis_primary"] = (1, 0, 0)
    j["limit_min"], j["limit_max"] = 0.0, 1.0
    j["impulse"][0, 0] = 0.2 if side == 0 else 0.0
    ob, oj = _step(b, j)
    if side == 0:
        assert oj["impulse"][0, 0] == 0 and np.all(ob["linear_velocity"][0] == 0)
        return
    erp, soft = _spring(float(DT))
    over = x - 1.0 if side > 0 else -x
    lam = side * (over - 0.005) * erp / (1.0 + soft)  # unadjustedError > 0 above the maximum
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(ob["linear_velocity"][0], (-lam, 0, 0), rtol=1e-4, atol=1e-9)
    assert np.sign(ob["linear_velocity"][0, 0]) == -side


def test_prismatic_limit_follows_the_flag():
    """PrismaticJoint's LinearAxisLimit (PrismaticJoint.cs:53-60) acts only when
    the record's LIMIT_ACTIVE flag is set; its impulse is record entry 5."""
    b = _body((1.5, 0, 0))
    j = _joint(N.JOINT_PRISMATIC, -1, 0)
    j["basis_primary"] = (1, 0, 0)
    j["basis_x"], j["test_axis"] = (0, 0, -1), (0, 1, 0)
    j["orientation_a"] = j["orientation_b"] = (0, 0, 0, 1)
    j["limit_min"], j["limit_max"] = 0.0, 1.0
    _, off = _step(b, j)
    assert off["impulse"][0, 5] == 0
    j["flags"] |= N.JOINT_LIMIT_ACTIVE
    ob, on = _step(b, j)
    erp, soft = _spring(float(DT))
    np.testing.assert_allclose(on["impulse"][0, 5], (0.5 - 0.005) * erp / (1.0 + soft), rtol=1e-4)
    assert ob["linear_velocity"][0, 0] < 0


def _ellipse_swing_x(theta, max_x=0.3, max_y=0.5):
    """B turned by theta about the world x axis; its twist axis is its local z.
    A is the world, with the basis z (primary), x, y."""
    b = _body((0, 0, 0), quat=(np.sin(theta / 2), 0, 0, np.cos(theta / 2)))
    j = _joint(N.JOINT_ELLIPSE_SWING_LIMIT, -1, 0)
    j["axis_a"], j["constrained_1"], j["constrained_2"] = (0, 0, 1), (1, 0, 0), (0, 1, 0)
    j["axis_b"] = (0, 0, 1)
    j["limit_min"], j["limit_max"] = max_x, max_y
    return b, j


def test_ellipse_swing_limit_inside_is_off():
    b, j = _ellipse_swing_x(0.2)
    j["impulse"][0, 0] = -0.3
    ob, oj = _step(b, j)
    assert oj["impulse"][0, 0] == 0 and np.all(ob["angular_velocity"][0] == 0)


def test_ellipse_swing_limit_closed_form():
    """EllipseSwingLimit (EllipseSwingLimit.cs:162-357): swung 0.4 rad about x
    against a 0.3 rad x-semi-axis: error maxY^2 (theta^2 - maxX^2), jacobian
    A = (2 angleX / maxX^2) x with angleX = -theta, a non-positive impulse
    that turns B back about -x."""
    theta, mx, my = 0.4, 0.3, 0.5
    b, j = _ellipse_swing_x(theta, mx, my)
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    error = my * my * (theta * theta - mx * mx) - 0.005
    t = 2 * theta / (mx * mx)  # |jacobian|
    lam = -(error * erp) / (soft + 2.0 * t * t)  # I_xx = 2
    assert oj["impulse"][0, 0] < 0
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(ob["angular_velocity"][0], (2.0 * t * lam, 0, 0), rtol=1e-4, atol=1e-8)


def test_ellipse_swing_limit_clamps_its_angles():
    """MaximumAngleX / Y setters clamp to [BigEpsilon, pi] (EllipseSwingLimit.cs:57-68)."""
    b, j = _ellipse_swing_x(0.4, 5.0, 0.5)
    _, oj = _step(b, j)
    b, j2 = _ellipse_swing_x(0.4, np.pi, 0.5)
    _, oj2 = _step(b, j2)
    assert oj["impulse"][0, 0] == oj2["impulse"][0, 0] == 0


def test_swivel_hinge_angular_to_world_closed_form():
    """SwivelHingeAngularJoint (SwivelHingeAngularJoint.cs:193-270): the world's
    hinge axis x against B's twist axis y turned by phi about z: error
    -sin(phi), jacobian A = z, an unclamped impulse whose bias is subtracted."""
    phi = 0.1
    b = _body((0, 0, 0), quat=_rot_z(phi))
    j = _joint(N.JOINT_SWIVEL_HINGE_ANGULAR, -1, 0)
    j["axis_a"], j["axis_b"] = (1, 0, 0), (0, 1, 0)
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    lam = np.sin(phi) * erp / (soft + 4.0)  # I_zz = 4, jacobianB = -z
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(ob["angular_velocity"][0], (0, 0, -4.0 * lam), rtol=1e-4, atol=1e-8)
    g = _joint(N.JOINT_SWIVEL_HINGE, -1, 0)  # ball socket at B's centre first: it does nothing here
    g["axis_a"], g["axis_b"] = (1, 0, 0), (0, 1, 0)
    _, og = _step(b, g)
    assert np.all(og["impulse"][0, :3] == 0)
    assert og["impulse"][0, 3] == oj["impulse"][0, 0]


def _motor(jtype, servo=False, goal=0.0, goal_velocity=0.0, max_force=np.finfo(np.float32).max):
    j = _joint(jtype, -1, 0)
    j["flags"] |= N.JOINT_SERVO if servo else 0
    j["limit_min"], j["limit_max"] = goal, goal_velocity
    j["margin"] = 0.0001                 # velocity motor softness
    j["bounciness"] = 0.0                # servo base corrective speed
    j["bounce_velocity_threshold"] = max_force
    return j


@pytest.mark.parametrize("max_force,expect", [(np.finfo(np.float32).max, None), (12.0, 0.2)])
def test_revolute_velocity_motor_closed_form(max_force, expect):
    """RevoluteMotor in velocity mode (RevoluteMotor.cs:243-340): goal 2 rad/s
    about z; its bias is subtracted, its softness is 0.0001 / dt, and the
    impulse is clamped to the maximum force times dt."""
    b = _body((0, 0, 0))
    j = _motor(N.JOINT_REVOLUTE_MOTOR, goal_velocity=2.0, max_force=max_force)
    j["basis_primary"], j["basis_x"], j["test_axis"] = (0, 0, 1), (1, 0, 0), (1, 0, 0)
    ob, oj = _step(b, j)
    lam = -2.0 / (0.0001 * 60 + 4.0)  # I_zz = 4, jacobian B = -z
    if expect is not None:
        lam = -expect                    # 12 * dt
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(ob["angular_velocity"][0], (0, 0, -4.0 * lam), rtol=1e-4, atol=1e-8)


def test_linear_axis_motors_closed_form():
    """LinearAxisMotor (LinearAxisMotor.cs:244-368): the velocity motor's bias
    is the negated goal velocity; the servo's is the error (separation less
    the goal) times the error reduction, pushing B back to the goal."""
    b = _body((0, 0, 0))
    j = _motor(N.JOINT_LINEAR_AXIS_MOTOR, goal_velocity=3.0)
    j["basis_primary"] = (1, 0, 0)
    ob, oj = _step(b, j)
    lam = -3.0 / (1.0 + 0.0001 * 60)
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(ob["linear_velocity"][0], (-lam, 0, 0), rtol=1e-4, atol=1e-9)
    b = _body((1.2, 0, 0))
    j = _motor(N.JOINT_LINEAR_AXIS_MOTOR, servo=True, goal=1.0)
    j["basis_primary"] = (1, 0, 0)
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    lam = 0.2 * erp / (1.0 + soft)
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(ob["linear_velocity"][0], (-lam, 0, 0), rtol=1e-4, atol=1e-9)


def test_twist_servo_motor_closed_form():
    """TwistMotor as a servo (TwistMotor.cs:182-253): turned 0.3 about z with
    goal 0, the distance from the goal is -0.3; jacobian B = z, and the
    positive-bias solve turns B back."""
    b, j0 = _twist_limit_z(0.3, 0, 0)
    j = _motor(N.JOINT_TWIST_MOTOR, servo=True, goal=2 * np.pi)  # wraps to 0
    for f in ("axis_a", "axis_b", "constrained_1", "constrained_2", "basis_x"):
        j[f] = j0[f]
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    lam = -0.3 * erp / (soft + 4.0)
    np.testing.assert_allclose(oj["impulse"][0, 0], lam, rtol=1e-4)
    np.testing.assert_allclose(ob["angular_velocity"][0], (0, 0, 4.0 * lam), rtol=1e-4, atol=1e-8)


def _speed_limit(jtype, max_speed, max_force=np.finfo(np.float32).max):
    j = _joint(jtype, 0, -1)
    j["limit_min"], j["limit_max"], j["margin"] = max_speed, max_force, 0.00001
    return j


@pytest.mark.parametrize("max_force,scale", [(np.finfo(np.float32).max, None), (60.0, 1.0)])
def test_maximum_linear_speed_closed_form(max_force, scale):
    """MaximumLinearSpeedConstraint (MaximumLinearVelocityConstraint.cs:138-193):
    speed 5 against a maximum of 2 is cut by (5 - 2) / 5 of the velocity times
    the effective mass 1 / (1/m + softness/dt); a maximum force scales the
    accumulated impulse to force * dt."""
    b = _body((0, 0, 0))
    b["linear_velocity"] = (3.0, 4.0, 0.0)
    ob, oj = _step(b, _speed_limit(N.JOINT_MAXIMUM_LINEAR_SPEED, 2.0, max_force))
    imp = np.array([3.0, 4.0, 0.0]) * (-3.0 / 5.0) / (1.0 + 0.00001 * 60)
    if scale is not None:
        imp = imp / np.linalg.norm(imp) * scale  # 60 * dt
    np.testing.assert_allclose(oj["impulse"][0, :3], imp, rtol=1e-4, atol=1e-7)
    np.testing.assert_allclose(ob["linear_velocity"][0], np.array([3.0, 4.0, 0.0]) + imp, rtol=1e-4)


def test_maximum_speeds_below_limit_and_angular():
    """Below the maximum nothing acts and the stale impulse is cleared (no warm
    start, :195-199); the angular form uses the inverse of (I^-1 + softness/dt)."""
    b = _body((0, 0, 0))
    b["linear_velocity"] = (1.0, 0.0, 0.0)
    j = _speed_limit(N.JOINT_MAXIMUM_LINEAR_SPEED, 2.0)
    j["impulse"][0, :3] = (0.5, 0.5, 0.5)
    ob, oj = _step(b, j)
    assert np.all(oj["impulse"][0, :3] == 0)
    np.testing.assert_array_equal(ob["linear_velocity"][0], (1.0, 0.0, 0.0))
    b = _body((0, 0, 0))
    b["angular_velocity"] = (0.0, 0.0, 10.0)
    ob, oj = _step(b, _speed_limit(N.JOINT_MAXIMUM_ANGULAR_SPEED, 4.0))
    imp_z = -6.0 / (4.0 + 0.00001 * 60)
    np.testing.assert_allclose(oj["impulse"][0, 2], imp_z, rtol=1e-4)
    np.testing.assert_allclose(ob["angular_velocity"][0, 2], 10.0 + 4.0 * imp_z, rtol=1e-4)


def test_plane_slider_is_its_point_on_plane_joint():
    """PlaneSliderJoint (PlaneSliderJoint.cs:48-69) with its limits and motors
    inactive, as constructed: a group of its point on plane joint alone."""
    b = _body((0.3, 0.1, -0.2))
    j = _joint(N.JOINT_POINT_ON_PLANE, -1, 0)
    j["axis_a"] = (0, 1, 0)
    g = j.copy()
    g["type"] = N.JOINT_PLANE_SLIDER
    ob, oj = _step(b, j)
    og_b, og = _step(b, g)
    assert og["impulse"][0, 0] == oj["impulse"][0, 0] != 0
    np.testing.assert_array_equal(og_b["linear_velocity"], ob["linear_velocity"])


def _angular_motor(servo=False):
    j = _motor(N.JOINT_ANGULAR_MOTOR, servo=servo)
    j["axis_a"], j["constrained_1"], j["constrained_2"] = (0, 0, 1), (1, 0, 0), (0, 1, 0)
    j["orientation_a"] = (0, 0, 0, 1)  # servo goal: the identity relative orientation
    return j


def test_angular_velocity_motor_closed_form():
    """AngularMotor in velocity mode (AngularMotor.cs:203-312): goal (0, 0, 2)
    in the basis; the impulse is (I_A^-1 + I_B^-1 + softness/dt)^-1 times
    (w_B - w_A - bias), applied to A and negated on B."""
    b = _body((0, 0, 0))
    j = _angular_motor()
    j["anchor_a"] = (0, 0, 2.0)
    ob, oj = _step(b, j)
    lam = -2.0 / (4.0 + 0.0001 * 60)
    np.testing.assert_allclose(oj["impulse"][0, :3], (0, 0, lam), rtol=1e-4, atol=1e-8)
    np.testing.assert_allclose(ob["angular_velocity"][0], (0, 0, -4.0 * lam), rtol=1e-4, atol=1e-8)


def test_angular_servo_motor_closed_form():
    """AngularMotor as a servo: B turned 0.2 about z from the goal (identity in
    a world basis) gets the bias -(0.2 erp) about z and turns back."""
    b = _body((0, 0, 0), quat=_rot_z(0.2))
    ob, oj = _step(b, _angular_motor(servo=True))
    erp, soft = _spring(float(DT))
    lam = 0.2 * erp / (4.0 + soft)
    np.testing.assert_allclose(oj["impulse"][0, :3], (0, 0, lam), rtol=1e-4, atol=1e-8)
    np.testing.assert_allclose(ob["angular_velocity"][0], (0, 0, -4.0 * lam), rtol=1e-4, atol=1e-8)


@pytest.mark.parametrize("servo", [False, True])
def test_single_entity_angular_motor_closed_form(servo):
    """SingleEntityAngularMotor (SingleEntityAngularMotor.cs:117-218) on body A:
    velocity goal (0, 0, 2) in its basis, or a servo back from 0.2 rad about z
    to the identity goal; lambda = (I^-1 + softness/dt)^-1 (bias - w)."""
    b = _body((0, 0, 0), quat=_rot_z(0.2) if servo else (0, 0, 0, 1))
    j = _angular_motor(servo=servo)
    j["type"], j["body_a"], j["body_b"] = N.JOINT_SINGLE_ENTITY_ANGULAR_MOTOR, 0, -1
    j["axis_a"], j["constrained_1"], j["constrained_2"] = (0, 0, 1), (1, 0, 0), (0, 1, 0)
    j["anchor_a"] = (0, 0, 2.0)
    ob, oj = _step(b, j)
    if servo:
        erp, soft = _spring(float(DT))
        lam = -0.2 * erp / (4.0 + soft)
    else:
        lam = 2.0 / (4.0 + 0.0001 * 60)
    np.testing.assert_allclose(oj["impulse"][0, :3], (0, 0, lam), rtol=1e-4, atol=1e-8)
    np.testing.assert_allclose(ob["angular_velocity"][0], (0, 0, 4.0 * lam), rtol=1e-4, atol=1e-8)


def _linear_motor(servo=False):
    j = _motor(N.JOINT_SINGLE_ENTITY_LINEAR_MOTOR, servo=servo)
    j["body_a"], j["body_b"] = 0, -1
    return j


def test_single_entity_linear_motor_closed_form():
    """SingleEntityLinearMotor (SingleEntityLinearMotor.cs:180-268): the centre
    driven at 1 m/s along x, then as a servo towards (0.5, 0, 0); at the goal
    the servo keeps the softness its record carries (impulse [3])."""
    b = _body((0, 0, 0))
    j = _linear_motor()
    j["axis_a"] = (1.0, 0, 0)
    ob, oj = _step(b, j)
    lam = 1.0 / (1.0 + 0.0001 * 60)
    np.testing.assert_allclose(oj["impulse"][0, :3], (lam, 0, 0), rtol=1e-4, atol=1e-8)
    np.testing.assert_allclose(ob["linear_velocity"][0], (lam, 0, 0), rtol=1e-4, atol=1e-8)
    j = _linear_motor(servo=True)
    j["anchor_b"] = (0.5, 0, 0)
    ob, oj = _step(b, j)
    erp, soft = _spring(float(DT))
    lam = 0.5 * erp / (1.0 + soft)
    np.testing.assert_allclose(oj["impulse"][0, :3], (lam, 0, 0), rtol=1e-4, atol=1e-8)
    np.testing.assert_allclose(oj["impulse"][0, 3], soft, rtol=1e-5)
    b["linear_velocity"] = (1.0, 0, 0)
    j = _linear_motor(servo=True)
    j["impulse"][0, 3] = 0.5  # at the goal: this softness stays
    ob, oj = _step(b, j)
    np.testing.assert_allclose(oj["impulse"][0, :3], (-1.0 / 1.5, 0, 0), rtol=1e-4, atol=1e-8)
    assert oj["impulse"][0, 3] == np.float32(0.5)


SINGLE_ENTITY = {N.JOINT_MAXIMUM_LINEAR_SPEED, N.JOINT_MAXIMUM_ANGULAR_SPEED, N.JOINT_SINGLE_ENTITY_ANGULAR_MOTOR,
                 N.JOINT_SINGLE_ENTITY_LINEAR_MOTOR}


@pytest.mark.parametrize("jtype", range(1, 30))
def test_every_joint_type_steps_in_the_oracle(jtype):
    """Every record type of the header builds its oracle object and steps: two
    moving bodies (or one, for the single-entity types) and the impulses stay
    finite."""
    a = _body((0, 0, 0))
    b = _body((0.1, -0.9, 0.05), quat=_rot_z(0.3))
    a["linear_velocity"], b["angular_velocity"] = (0.5, 0, 0), (0, 1.0, 2.0)
    bodies = np.concatenate([a, b])
    j = _joint(jtype, 0, -1 if jtype in SINGLE_ENTITY else 1)
    j["anchor_a"], j["anchor_b"] = (0, -0.5, 0), (0, 0.4, 0)
    j["axis_a"] = j["axis_b"] = j["basis_primary"] = (1, 0, 0)
    j["constrained_1"], j["constrained_2"] = (0, 1, 0), (0, 0, 1)
    j["basis_x"], j["test_axis"] = (0, 1, 0), (0, 1, 0)
    j["orientation_a"] = j["orientation_b"] = (0, 0, 0, 1)
    j["limit_min"], j["limit_max"] = 0.1, 0.3
    j["impulse"][0, :4] = 0.01
    o = oracle.OracleSpace(_settings(5), bodies, np.zeros(0, N.MANIFOLD_DTYPE), j)
    o.step(DT, N.STEP_ALL, 3)
    ob, oj = o.get_bodies(), o.get_constraints()[1]
    o.close()
    assert np.all(np.isfinite(ob["linear_velocity"])) and np.all(np.isfinite(ob["angular_velocity"]))
    assert np.all(np.isfinite(oj["impulse"]))
