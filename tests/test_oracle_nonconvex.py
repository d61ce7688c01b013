"""Closed-form pins of the oracle's NonConvexContactManifoldConstraint: one
sphere on a static ground with a single contact, its penetration child then
its ContactFrictionConstraint (ContactFrictionConstraint.cs:95-299)."""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300.solver import default_settings

DT = np.float32(1 / 60)
R = np.float32(0.5)
MU = np.float32(0.5)


def _sphere_on_ground(vx=1.0, vy=-1.0, direction=(0.0, 0.0, 0.0), friction_impulse=0.0, flags=None):
    """Ground (kinematic, body A) and a unit-mass sphere of radius R (body B)
    touching at the origin; the contact normal points from A to B."""
    bodies = np.zeros(2, N.BODY_DTYPE)
    for b in bodies:
        b["orientation"] = (0, 0, 0, 1)
    bodies[0]["position"] = (0, -1, 0)
    bodies[1]["position"] = (0, R, 0)
    bodies[1]["is_dynamic"] = 1
    bodies[1]["inverse_mass"] = 1
    inv = np.float32(2.5) / (R * R)  # SphereShape: I = 2/5 m r^2 (InertiaTensorScale folded in)
    bodies[1]["local_inverse_inertia"] = (inv, 0, 0, 0, inv, 0, 0, 0, inv)
    bodies[1]["linear_velocity"] = (vx, vy, 0)
    m = np.zeros(1, N.MANIFOLD_DTYPE)
    m[0]["body_a"], m[0]["body_b"], m[0]["contact_count"] = 0, 1, 1
    m[0]["flags"] = N.MANIFOLD_ACTIVE | N.MANIFOLD_SOLVER_RULE | N.MANIFOLD_NONCONVEX if flags is None else flags
    m[0]["kinetic_friction"] = MU
    m[0]["static_friction"] = np.float32(0.8)
    c = m[0]["contacts"][0]
    c["normal"] = (0, 1, 0)
    c["friction_direction"] = direction
    c["friction_impulse"] = friction_impulse
    m[0]["contacts"][0] = c
    return bodies, m


def _solve_once(bodies, m):
    s = default_settings()
    s["iteration_limit"] = 1
    s["gravity"] = (0, 0, 0)
    o = oracle.OracleSpace(s, bodies, m)
    o.step(DT, N.STEP_SOLVE, 1)
    b = o.get_bodies()
    mo, _ = o.get_constraints()
    solves = o.last_child_solves()
    o.close()
    return b, mo, solves


def test_sliding_sphere_known_answer():
    """Penetration: lambda = -rv / (1 + softness) with rv = -1 (approach),
    softness = 0.001 * 60.  Friction: direction -x (the relative velocity A - B),
    kinetic (|v| = 1 > 0.2), effective mass 1 + r^2 (2.5 / r^2) = 3.5, so
    lambda = 1 * (-1 / 3.5) inside the cone mu * 1/1.06; it stops the contact
    point: v_x = 1 - 2/7, w_z = -(2/7) r (2.5 / r^2)."""
    b, mo, solves = _solve_once(*_sphere_on_ground())
    f32 = np.float32
    softness = f32(f32(f32(0.001) * f32(1)) * f32(f32(1) / DT))
    pen = f32(f32(-1) * f32(f32(-1) / f32(softness + f32(1))))
    fric = f32(f32(1) * f32(f32(-1) / f32(3.5)))
    c = mo[0]["contacts"][0]
    assert c["penetration_impulse"] == pytest.approx(float(pen), rel=1e-6)
    assert c["friction_impulse"] == pytest.approx(float(fric), rel=1e-6)
    np.testing.assert_allclose(c["friction_direction"], (-1, 0, 0), atol=0)
    v, w = b[1]["linear_velocity"], b[1]["angular_velocity"]
    assert v[0] == pytest.approx(1 - 2 / 7, rel=1e-6)
    assert v[1] == pytest.approx(-1 + float(pen), rel=1e-5)
    assert w[2] == pytest.approx(-(2 / 7) * 2.5 / float(R), rel=1e-6)
    # the contact point no longer slides: v + w x rb with rb = (0, -r, 0)
    assert v[0] + w[2] * float(R) == pytest.approx(0, abs=1e-6)
    assert solves == 2  # one penetration and one friction child; no sliding or twist children
    assert mo[0]["sliding_impulse"][0] == 0 and mo[0]["twist_impulse"] == 0


def test_friction_cone_clamps():
    """Fast sliding with a small normal impulse: |lambda| is clamped to
    mu * penetration impulse."""
    b, mo, _ = _solve_once(*_sphere_on_ground(vx=10.0, vy=-0.1))
    c = mo[0]["contacts"][0]
    assert c["friction_impulse"] == pytest.approx(-float(MU) * float(c["penetration_impulse"]), rel=1e-6)


def test_resting_contact_without_direction_has_no_friction_child():
    """No tangential velocity and no kept direction: the friction child gives
    up for the step (isActiveInSolver = false), only the penetration solves."""
    b, mo, solves = _solve_once(*_sphere_on_ground(vx=0.0))
    assert solves == 1
    assert mo[0]["contacts"][0]["friction_impulse"] == 0
    assert b[1]["linear_velocity"][0] == 0


def test_kept_direction_uses_static_friction():
    """No tangential velocity but a kept direction (+x) and a warm-start
    impulse: the child stays active with static friction; the warm start
    pushes the sphere along +x times the impulse and the solve takes it back
    within mu_static * penetration impulse."""
    bodies, m = _sphere_on_ground(vx=0.0, direction=(1.0, 0.0, 0.0), friction_impulse=0.3)
    b, mo, solves = _solve_once(bodies, m)
    assert solves == 2
    c = mo[0]["contacts"][0]
    np.testing.assert_allclose(c["friction_direction"], (1, 0, 0), atol=0)
    assert abs(c["friction_impulse"]) <= 0.8 * c["penetration_impulse"] * (1 + 1e-6)


def test_convex_flag_off_gives_sliding_friction():
    """The same pair without NONCONVEX is a convex manifold: sliding and
    twist friction, no contact friction."""
    bodies, m = _sphere_on_ground(flags=N.MANIFOLD_ACTIVE | N.MANIFOLD_SOLVER_RULE)
    b, mo, solves = _solve_once(bodies, m)
    assert solves == 3
    assert mo[0]["contacts"][0]["friction_impulse"] == 0
    assert mo[0]["sliding_impulse"][0] != 0
