"""Joints on the device against the oracle: BallSocketJoint, SwingLimit,
RevoluteAngularJoint, RevoluteLimit and the RevoluteJoint group, alone and
mixed with contact manifolds in one colouring (the chains workload)."""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, default_settings

from joint_records import MOTORS, NEW_TYPES, SPEED_LIMITS, convert as _convert
from parity import DT, LONG_TOL, STEP_TOL, Pair

pytestmark = pytest.mark.gpu


def _settings(iterations=15):
    s = default_settings()
    s["iteration_limit"] = iterations
    return s


def _small_chains(seed=5, chains=48, links=16, loose=300):
    return scenes.make_chain(chains=chains, links=links, loose_bodies=loose, seed=seed,
                             region=np.array([30.0, 12.0, 30.0], np.float32))


def test_chain_colouring_mixes_joints_and_manifolds(gpu_context):
    b, m, j = _small_chains()
    assert len(j) and len(m)
    sp = GpuSpace(gpu_context, b, m, j)
    col, order, k = sp.colouring()
    col2, order2, k2 = oracle.colour(b, m, j)
    assert k == k2
    np.testing.assert_array_equal(col, col2)
    np.testing.assert_array_equal(order, order2)
    # joints and manifolds share colours: the sweep is mixed
    jc, mc = set(col[:len(j)]), set(col[len(j):])
    assert jc & mc
    sp.close()


def test_chains_every_step(gpu_context):
    b, m, j = _small_chains()
    p = Pair(gpu_context, b, m, j, settings=_settings())
    for step in range(8):
        p.step()
        errs, exact = p.compare()
        for k, v in errs.items():
            assert v <= STEP_TOL, (step, k, v)
        assert exact, (step, errs)
    p.close()


def test_chains_sixty_steps(gpu_context):
    b, m, j = _small_chains(seed=6)
    p = Pair(gpu_context, b, m, j, settings=_settings())
    p.step(steps=60)
    errs, exact = p.compare()
    for k, v in errs.items():
        assert v <= LONG_TOL, (k, v)
    assert exact, errs
    p.close()


def test_chains_persistent_mode(gpu_context):
    b, m, j = _small_chains(seed=7, chains=16)
    p = Pair(gpu_context, b, m, j, settings=_settings(), mode=N.MODE_PERSISTENT)
    p.step(steps=10)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


@pytest.mark.parametrize("kind", ["ball", "swing", "angular", "revolute_limit", "revolute"])
def test_each_joint_type_alone(gpu_context, kind):
    """Every record type on its own, between two bodies and to the world, with
    limits started inside and outside their range and stale impulses."""
    b, m, j = _small_chains(seed=11, chains=24, loose=0)
    t = j["type"]
    if kind == "ball":
        keep = t == N.JOINT_BALL_SOCKET
    elif kind == "swing":
        keep = (t == N.JOINT_SWING_LIMIT) | ((t == N.JOINT_BALL_SOCKET) & (j["body_a"] == -1))
    elif kind == "angular":
        keep = t == N.JOINT_REVOLUTE
        j = j.copy()
        j["type"][keep] = N.JOINT_REVOLUTE_ANGULAR
    elif kind == "revolute_limit":
        keep = t == N.JOINT_REVOLUTE
        j = j.copy()
        j["type"][keep] = N.JOINT_REVOLUTE_LIMIT
        j["impulse"][keep, 0:2] = j["impulse"][keep, 5:7]
    else:
        keep = (t == N.JOINT_REVOLUTE) | (t == N.JOINT_BALL_SOCKET)
    jj = j[keep].copy()
    rng = np.random.default_rng(3)
    jj["impulse"] = rng.uniform(0, 0.05, jj["impulse"].shape).astype(np.float32)
    p = Pair(gpu_context, b, m, jj, settings=_settings())
    for step in range(4):
        p.step()
        errs, exact = p.compare()
        assert exact, (kind, step, errs)
    p.close()


def test_inactive_joints_and_world_anchors(gpu_context):
    """IsActive off on some joints and on revolute limits; both connections
    kinematic on others: they never enter the solver."""
    b, m, j = _small_chains(seed=12, chains=12, loose=40)
    j = j.copy()
    j["flags"][::5] &= ~np.uint32(N.JOINT_ACTIVE)
    rev = np.flatnonzero(j["type"] == N.JOINT_REVOLUTE)
    j["flags"][rev[::2]] &= ~np.uint32(N.JOINT_LIMIT_ACTIVE)
    b = b.copy()
    b["is_dynamic"][len(b) - 3:] = 0  # the last chain's tail becomes kinematic
    b["inverse_mass"][len(b) - 3:] = 0
    p = Pair(gpu_context, b, m, j, settings=_settings())
    p.step(steps=6)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


def test_joint_records_roundtrip_and_checks(gpu_context):
    b, m, j = _small_chains(seed=13, chains=4, loose=0)
    j = j.copy()
    j["impulse"] = np.random.default_rng(1).normal(size=j["impulse"].shape).astype(np.float32)
    sp = GpuSpace(gpu_context, b, m, j)
    _, back = sp.download_constraints(joints=j.copy())
    used = {N.JOINT_BALL_SOCKET: 3, N.JOINT_SWING_LIMIT: 1, N.JOINT_REVOLUTE: 7}
    for t, n in used.items():
        sel = j["type"] == t
        np.testing.assert_array_equal(back["impulse"][sel, :n], j["impulse"][sel, :n])
    bad = j.copy()
    bad["type"][0] = 42
    with pytest.raises(N.BepuError):
        sp.upload_constraints(m, bad)
    bad = j.copy()
    bad["spring_stiffness"][1] = 0
    bad["spring_damping"][1] = 0
    with pytest.raises(N.BepuError):
        sp.upload_constraints(m, bad)
    bad = j.copy()
    bad["body_b"][2] = len(b)
    with pytest.raises(N.BepuError):
        sp.upload_constraints(m, bad)
    sp.close()


def test_chains_full_size_two_steps(gpu_context):
    """The full mixed workload (8,192 chains of 16 capsules, 20,000 loose
    bodies, 15 iterations) against the oracle for two steps."""
    b, m, j = scenes.chains_8k()
    p = Pair(gpu_context, b, m, j, settings=_settings())
    p.step(steps=2)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


@pytest.mark.parametrize("policy", [(0, 1024, 4096, 64, 0), (1, 1024, 4096, 16, 0), (1, 1024, 4096, 256, 64)])
def test_chains_in_island_groups(gpu_context, policy):
    """Joint islands run whole steps inside island-group CTAs (or on the sweep
    path with groups off); every policy gives the oracle's bits."""
    b, m, j = _small_chains(seed=14, chains=20)
    p = Pair(gpu_context, b, m, j, settings=_settings(), group_policy=policy)
    p.step(steps=5)
    errs, exact = p.compare()
    assert exact, (policy, errs)
    if policy[0]:
        # chains and loose stacks are small islands: the step is group launches alone,
        # one per group kind (shared or global lanes, with or without joints)
        assert p.gpu.last_step_launches() <= 4
    p.close()


def test_weld_no_rotation_distance_every_step(gpu_context):
    b, m, j = _small_chains(seed=21)
    j = _convert(b, j, NEW_TYPES, 21)
    p = Pair(gpu_context, b, m, j, settings=_settings())
    for step in range(8):
        p.step()
        errs, exact = p.compare()
        assert exact, (step, errs)
    p.close()


@pytest.mark.parametrize("jtype", NEW_TYPES)
def test_each_new_type_alone_with_stale_impulses(gpu_context, jtype):
    b, m, j = _small_chains(seed=22, chains=16, loose=60)
    j = _convert(b, j, (jtype,), 22)
    j["impulse"] = np.random.default_rng(5).uniform(0, 0.05, j["impulse"].shape).astype(np.float32)
    if jtype in SPEED_LIMITS:  # spinning links, so the angular speed limits have work too
        b = b.copy()
        dyn = b["is_dynamic"] == 1
        b["angular_velocity"][dyn] = np.random.default_rng(6).uniform(-2, 2, (int(dyn.sum()), 3))
    p = Pair(gpu_context, b, m, j, settings=_settings())
    for step in range(5):
        p.step()
        errs, exact = p.compare()
        assert exact, (jtype, step, errs)
        if step == 0:  # speed limits start from zero each step: the first one shows their work
            first = p.oracle.get_constraints()[1]["impulse"]
    limit_entry = {N.JOINT_TWIST_LIMIT: 0, N.JOINT_LINEAR_AXIS_LIMIT: 0, N.JOINT_ELLIPSE_SWING_LIMIT: 0,
                   N.JOINT_PRISMATIC: 5, N.JOINT_LINE_SLIDER: 4, N.JOINT_REVOLUTE_MOTOR: 0,
                   N.JOINT_TWIST_MOTOR: 0, N.JOINT_LINEAR_AXIS_MOTOR: 0, N.JOINT_MAXIMUM_LINEAR_SPEED: 0,
                   N.JOINT_MAXIMUM_ANGULAR_SPEED: 2, N.JOINT_ANGULAR_MOTOR: 0,
                   N.JOINT_SINGLE_ENTITY_ANGULAR_MOTOR: 0, N.JOINT_SINGLE_ENTITY_LINEAR_MOTOR: 0}
    if jtype in limit_entry:  # some limits pushed: impulses that are new and nonzero
        e = limit_entry[jtype]
        e = slice(0, 3) if jtype in SPEED_LIMITS + (N.JOINT_ANGULAR_MOTOR, N.JOINT_SINGLE_ENTITY_ANGULAR_MOTOR,
                                                    N.JOINT_SINGLE_ENTITY_LINEAR_MOTOR) \
            else slice(e, e + 1)
        got = (first if jtype in SPEED_LIMITS else p.oracle.get_constraints()[1]["impulse"])[:, e]
        assert np.count_nonzero(np.any((got != j["impulse"][:, e]) & (got != 0), axis=1)) > 0
    p.close()


@pytest.mark.parametrize("policy,mode", [(None, N.MODE_GRAPH), ((0, 1024, 4096, 64, 0), N.MODE_GRAPH),
                                         (None, N.MODE_PERSISTENT)])
def test_new_types_sixty_steps_every_path(gpu_context, policy, mode):
    b, m, j = _small_chains(seed=23, chains=20)
    j = _convert(b, j, NEW_TYPES, 23)
    p = Pair(gpu_context, b, m, j, settings=_settings(), group_policy=policy, mode=mode)
    p.step(steps=60)
    errs, exact = p.compare()
    assert exact, (policy, mode, errs)
    p.close()


def test_new_type_records_checked(gpu_context):
    b, m, j = _small_chains(seed=24, chains=2, loose=0)
    j = _convert(b, j, (N.JOINT_DISTANCE_LIMIT,), 24)
    bad = j.copy()
    bad["limit_min"][0], bad["limit_max"][0] = 2.0, 1.0
    with pytest.raises(N.BepuError):
        GpuSpace(gpu_context, b, m, bad)
    bad = _convert(b, j, (N.JOINT_DISTANCE,), 25)
    bad["limit_min"][1] = -1.0
    with pytest.raises(N.BepuError):
        GpuSpace(gpu_context, b, m, bad)


@pytest.mark.parametrize("jtype", [N.JOINT_TWIST_LIMIT, N.JOINT_SINGLE_ENTITY_LINEAR_MOTOR, N.JOINT_PRISMATIC,
                                   N.JOINT_ANGULAR_MOTOR, N.JOINT_REVOLUTE_MOTOR])
def test_added_types_resume_from_records(gpu_context, jtype):
    """Stepping, downloading the records (bodies and joints: impulses, a twist
    limit's last error, a linear motor's kept softness), uploading them into a
    new scene and stepping on continues bit for bit like the uninterrupted run."""
    b, m, j = _small_chains(seed=31, chains=12, loose=40)
    j = _convert(b, j, (jtype,), 31)
    gpu_context.set_settings(_settings())
    ref = GpuSpace(gpu_context, b, m, j)
    for _ in range(6):
        ref.step(float(DT))
    cut = GpuSpace(gpu_context, b, m, j)
    for _ in range(3):
        cut.step(float(DT))
    mb = cut.download_bodies(b.copy())
    mm, mj = cut.download_constraints(m.copy(), j.copy())
    again = GpuSpace(gpu_context, mb, mm, mj)
    for _ in range(3):
        again.step(float(DT))
    rb, ab = ref.download_bodies(b.copy()), again.download_bodies(b.copy())
    for f in ("position", "orientation", "linear_velocity", "angular_velocity"):
        np.testing.assert_array_equal(rb[f], ab[f], err_msg=f)
    np.testing.assert_array_equal(ref.download_constraints(m.copy(), j.copy())[1]["impulse"],
                                  again.download_constraints(m.copy(), j.copy())[1]["impulse"])
    for s in (ref, cut, again):
        s.close()


def test_added_type_mix_of_the_bench(gpu_context):
    """scenes.with_added_joint_types (the bench's added-types chains) against the
    oracle, on the island-group path and the sweep path."""
    b, m, j = _small_chains(seed=41, chains=30, loose=80)
    mixed = scenes.with_added_joint_types(b, j)
    assert len(set(mixed["type"].tolist())) == 10
    for policy in (None, (0, 1024, 4096, 64, 0)):
        p = Pair(gpu_context, b, m, mixed, settings=_settings(), group_policy=policy)
        p.step(steps=20)
        errs, exact = p.compare()
        assert exact, (policy, errs)
        p.close()
