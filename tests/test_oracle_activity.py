"""CPU pins of the oracle's activity state: the deactivation candidacy update
(SimulationIslandMember.UpdateDeactivationCandidacy, SimulationIslandMember.cs:53-164)
and the stabilization boost of the force update (EntityBase.cs:926-936), checked
against answers worked out here in float32 from the reference's statements."""
import math

import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300.solver import default_settings

f32 = np.float32
DT = f32(1 / 60)
G = f32(-9.81)


def _one_body(v=(0, 0, 0), w=(0, 0, 0), dynamic=True, activity=0, previous=0.0, time_below=0.0,
              q=(0, 0, 0, 1)):
    b = np.zeros(1, N.BODY_DTYPE)
    b["orientation"] = q
    b["linear_damping"] = 0.03
    b["angular_damping"] = 0.15
    b["linear_velocity"] = v
    b["angular_velocity"] = w
    b["is_dynamic"] = 1 if dynamic else 0
    if dynamic:
        b["inverse_mass"] = 1
        b["local_inverse_inertia"] = np.diag([6.0, 6.0, 6.0]).astype(np.float32).ravel()
    b["activity"] = activity
    b["previous_velocity"] = previous
    b["velocity_time_below_limit"] = time_below
    return b


def _run(b, flags, steps=1, settings=None):
    o = oracle.OracleSpace(default_settings() if settings is None else settings, b, np.zeros(0, N.MANIFOLD_DTYPE))
    o.step(DT, flags, steps)
    out = o.get_bodies()
    o.close()
    return out[0]


def _len2(v):
    v = [f32(x) for x in v]
    return f32(f32(f32(v[0] * v[0]) + f32(v[1] * v[1])) + f32(v[2] * v[2]))


def _factor(d):
    # (float)Math.Pow(MathHelper.Clamp(1 - d, 0, 1), dt)
    c = min(max(f32(f32(1) - d), f32(0)), f32(1))
    return f32(math.pow(float(c), float(DT)))


def test_stabilization_boost_known_answer():
    """A slowing body under the velocity limit: boost = 1 - sqrt(energy) / (2 limit);
    each damping becomes d + boost (1 - d) for this step (ModifyLinearDamping, EntityBase.cs:1205-1210)."""
    v0, w0 = (f32(0.01), f32(0.0), f32(-0.02)), (f32(0.0), f32(0.03), f32(0.0))
    b = _one_body(v0, w0, activity=N.BODY_SLOWING)
    out = _run(b, N.STEP_FORCES)
    v1 = [f32(0 + v0[0]), f32(f32(G * DT) + v0[1]), f32(0 + v0[2])]
    energy = f32(_len2(v1) + _len2(w0))
    assert energy < f32(f32(0.26) * f32(0.26))
    boost = f32(f32(1) - f32(math.sqrt(float(energy)) / float(f32(f32(2) * f32(0.26)))))
    lin = f32(f32(0.03) + f32(f32(0) + f32(boost * f32(f32(1) - f32(f32(0.03) + f32(0))))))
    ang = f32(f32(0.15) + f32(f32(0) + f32(boost * f32(f32(1) - f32(f32(0.15) + f32(0))))))
    fl, fa = _factor(lin), _factor(ang)
    want_v = np.array([f32(x * fl) for x in v1], np.float32)
    want_w = np.array([f32(x * fa) for x in w0], np.float32)
    np.testing.assert_array_equal(out["linear_velocity"], want_v)
    np.testing.assert_array_equal(out["angular_velocity"], want_w)
    # the boost only lasts the step: the plain factors are well above the boosted ones
    assert fl < _factor(f32(0.03)) and fa < _factor(f32(0.15))


@pytest.mark.parametrize("case", ["not_slowing", "disallowed", "setting_off", "fast"])
def test_no_boost(case):
    v0, w0 = (f32(0.01), f32(0.0), f32(-0.02)), (f32(0.0), f32(0.03), f32(0.0))
    activity, settings = N.BODY_SLOWING, default_settings()
    if case == "not_slowing":
        activity = 0
    elif case == "disallowed":
        activity |= N.BODY_NO_STABILIZATION
    elif case == "setting_off":
        settings["use_stabilization"] = 0
    else:
        v0 = (f32(0.5), f32(0.0), f32(0.0))
    out = _run(_one_body(v0, w0, activity=activity), N.STEP_FORCES, settings=settings)
    v1 = [f32(0 + v0[0]), f32(f32(G * DT) + v0[1]), f32(0 + v0[2])]
    np.testing.assert_array_equal(out["linear_velocity"], np.array([f32(x * _factor(f32(0.03))) for x in v1]))
    np.testing.assert_array_equal(out["angular_velocity"], np.array([f32(x * _factor(f32(0.15))) for x in w0]))


def _candidacy(v, w, dynamic, activity, previous, t, steps, limit=f32(0.26), minimum=f32(1)):
    """UpdateDeactivationCandidacy restated in float32 for a body whose velocity
    the steps do not change (candidacy stage only)."""
    velocity = f32(_len2(v) + _len2(w))
    always = bool(activity & N.BODY_ALWAYS_ACTIVE)
    slowing = bool(activity & N.BODY_SLOWING)
    cand = bool(activity & N.BODY_DEACTIVATION_CANDIDATE)
    t = f32(t)
    previous = f32(previous)
    for _ in range(steps):
        if dynamic or t <= 0:
            slowing = velocity <= previous
            if dynamic:
                t = f32(t + DT) if velocity < f32(limit * limit) else f32(0)
                if not always:
                    if not cand:
                        if t > minimum and slowing:
                            cand = True
                    elif t <= minimum:
                        cand, t = False, f32(0)
                else:
                    cand, t = False, f32(0)
            else:
                cand = velocity == 0 and not always
                if not cand:
                    t = f32(0)
                if cand:
                    t = f32(1) if t == 0 else (f32(0) if t < 0 else t)
                else:
                    t = f32(-1)
        previous = velocity
    flags = (activity & (N.BODY_ALWAYS_ACTIVE | N.BODY_NO_STABILIZATION)) | \
        (N.BODY_SLOWING if slowing else 0) | (N.BODY_DEACTIVATION_CANDIDATE if cand else 0)
    return flags, previous, t


@pytest.mark.parametrize("steps", [1, 2, 59, 60, 61, 62, 75])
def test_candidacy_of_a_slow_body(steps):
    """Below the velocity limit the time accumulates by dt; past one second of
    slowing the body becomes a deactivation candidate (SimulationIslandMember.cs:68-90)."""
    v, w = (0.0, 0.05, 0.0), (0.01, 0.0, 0.0)
    out = _run(_one_body(v, w), N.STEP_DEACTIVATION, steps)
    flags, previous, t = _candidacy(v, w, True, 0, 0.0, 0.0, steps)
    assert (int(out["activity"]), out["previous_velocity"], out["velocity_time_below_limit"]) == \
        (flags, previous, t)
    if steps >= 62:
        assert flags & N.BODY_DEACTIVATION_CANDIDATE


def test_candidate_that_speeds_up_is_reset():
    # a candidate above the limit: the time resets, and with it the candidacy
    b = _one_body((0.5, 0, 0), activity=N.BODY_DEACTIVATION_CANDIDATE | N.BODY_SLOWING, previous=0.1,
                  time_below=2.0)
    out = _run(b, N.STEP_DEACTIVATION)
    assert int(out["activity"]) == 0 and out["velocity_time_below_limit"] == 0
    assert out["previous_velocity"] == f32(f32(0.5) * f32(0.5))


def test_always_active_body_never_accumulates():
    b = _one_body((0.0, 0.05, 0.0), activity=N.BODY_ALWAYS_ACTIVE)
    out = _run(b, N.STEP_DEACTIVATION, 100)
    assert out["velocity_time_below_limit"] == 0
    assert int(out["activity"]) == N.BODY_ALWAYS_ACTIVE | N.BODY_SLOWING


@pytest.mark.parametrize("time_below,moving,always,steps", [
    (0.0, False, False, 1), (0.0, False, False, 3), (-1.0, False, False, 1), (-1.0, False, False, 2),
    (1.0, False, False, 2), (1.0, True, False, 1), (0.0, True, False, 1), (0.0, False, True, 2)])
def test_kinematic_time_flag(time_below, moving, always, steps):
    """A kinematic body's time field is an activity flag: -1 active, 0 active
    for one more step, 1 inactive (SimulationIslandMember.cs:102-122)."""
    v = (0.0, 0.0, 0.5) if moving else (0.0, 0.0, 0.0)
    activity = N.BODY_ALWAYS_ACTIVE if always else 0
    out = _run(_one_body(v, dynamic=False, activity=activity, time_below=time_below, previous=0.25),
               N.STEP_DEACTIVATION, steps)
    flags, previous, t = _candidacy(v, (0, 0, 0), False, activity, 0.25, time_below, steps)
    assert (int(out["activity"]), out["previous_velocity"], out["velocity_time_below_limit"]) == \
        (flags, previous, t)


def test_kinematic_position_update_follows_the_flag():
    """An inactive kinematic body is not integrated; an active one at rest is,
    which renormalises its orientation (EntityBase.cs:1124-1160)."""
    q = np.array([0.1, 0.2, 0.3, 0.9], np.float32)
    flags = N.STEP_DEACTIVATION | N.STEP_POSITIONS
    out = _run(_one_body(dynamic=False, time_below=1.0, q=q), flags)
    np.testing.assert_array_equal(out["orientation"], q)
    out = _run(_one_body(dynamic=False, time_below=-1.0, q=q), flags)  # -1 -> 0: still active this step
    inv = f32(1.0 / math.sqrt(float(_len2(q[:3]) + f32(q[3] * q[3]))))
    assert out["velocity_time_below_limit"] == 0
    np.testing.assert_array_equal(out["orientation"], (q + np.zeros(4, np.float32)) * inv)
