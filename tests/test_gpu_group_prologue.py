"""The island groups' split prologue (bepugpu_set_group_prologue = 1: the
refresh, the body updates and the prestep as grid-wide launches before the
group kernel, which copies the solve lanes into shared memory) against the
oracle, on every kind of group: shared and global solve lanes, convex and
NONCONVEX manifolds, joints of the classic and the added types, the narrow
phase, islands asleep and woken; and equal bit for bit to the in-kernel
prologue on the full 65,536-box pile."""
import numpy as np
import pytest

from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, default_settings, islands_of

from island_records import sleepy_pile, with_moving_kinematics
from parity import DT, Pair

pytestmark = pytest.mark.gpu

GROUPS = (1, 1024, 4096, 256, 0)
MIXED = (1, 24, 4096, 64, 0)


def _split_pair(ctx, b, m, j=None, policy=GROUPS, settings=None, shapes=None, mode=1):
    p = Pair(ctx, b, m, j, settings=settings, group_policy=policy, shapes=shapes)
    p.gpu.set_group_prologue(mode)
    return p


def _run_exact(p, chunks, steps, flags=N.STEP_ALL):
    for c in range(chunks):
        p.step(flags=flags, steps=steps)
        errs, exact = p.compare()
        assert exact, (c, errs)


@pytest.mark.parametrize("policy", [GROUPS, MIXED])
def test_pile_1k_and_towers(gpu_context, policy):
    """pile_1k is one island of 1,000 boxes (lanes in global memory under
    GROUPS, sweeps under MIXED); the towers are many small islands (lanes in
    shared memory)."""
    for b, m in (scenes.pile_1k()[:2], scenes.make_tower(1200, seed=17)[:2]):
        p = _split_pair(gpu_context, b, m, policy=policy)
        _run_exact(p, 3, 7)
        p.close()


@pytest.mark.parametrize("flags", [N.STEP_SOLVE, N.STEP_SOLVE | N.STEP_FORCES,
                                   N.STEP_ALL & ~N.STEP_REFRESH_CONTACTS & ~N.STEP_COLLIDE,
                                   N.STEP_ALL & ~N.STEP_DEACTIVATION & ~N.STEP_COLLIDE])
def test_stage_subsets(gpu_context, flags):
    b, m, _ = scenes.make_tower(800, seed=5)
    p = _split_pair(gpu_context, b, m, policy=MIXED)
    _run_exact(p, 2, 6, flags=flags)
    p.close()


def test_persistent_mode_with_sweeps(gpu_context):
    """Groups beside the colour sweeps of the persistent kernel."""
    b, m, _ = scenes.make_tower(1200, seed=19)
    p = Pair(gpu_context, b, m, group_policy=MIXED, mode=N.MODE_PERSISTENT)
    p.gpu.set_group_prologue(1)
    _run_exact(p, 3, 7)
    p.close()


def test_nonconvex_towers(gpu_context):
    b, m, _ = scenes.make_tower(600, seed=14, sphere_fraction=0.5)
    assert np.any(m["flags"] & N.MANIFOLD_NONCONVEX)
    p = _split_pair(gpu_context, b, m)
    _run_exact(p, 4, 5)
    gm, _ = p.gpu.download_constraints()
    om, _ = p.oracle.get_constraints()
    for f in ("friction_impulse", "friction_direction"):
        assert gm["contacts"][f].tobytes() == om["contacts"][f].tobytes(), f
    p.close()


@pytest.mark.parametrize("added", [False, True])
def test_chains(gpu_context, added):
    b, m, j = scenes.make_chain(chains=24, links=10, loose_bodies=80, seed=8,
                                region=np.array([30.0, 12.0, 30.0], np.float32))
    if added:
        j = scenes.with_added_joint_types(b, j)
    s = default_settings()
    s["iteration_limit"] = 15
    p = _split_pair(gpu_context, b, m, j, settings=s)
    _run_exact(p, 3, 10)
    p.close()


def test_narrow_phase(gpu_context):
    b, m, _, sh = scenes.make_pile(nx=6, ny=6, nz=6, narrow_phase=1, seed=21)
    p = _split_pair(gpu_context, b, m, shapes=sh)
    _run_exact(p, 3, 8, flags=N.STEP_ALL | N.STEP_COLLIDE)
    p.close()


def test_islands_asleep_and_woken(gpu_context):
    b, m, j = sleepy_pile(nx=6, ny=4, nz=6, ground_at=40)
    isl = islands_of(b, m, j)
    p = _split_pair(gpu_context, b, m, j)
    p.gpu.set_islands(isl)
    p.oracle.set_islands(isl)
    p.step(steps=140)
    errs, exact = p.compare()
    assert exact, errs
    flags, idx = p.gpu.get_islands()
    of, oi = p.oracle.get_islands()
    np.testing.assert_array_equal(flags, of)
    assert idx == oi and not np.any(flags & N.ISLAND_ACTIVE)
    sb = p.gpu.download_bodies(b.copy())
    sm, _ = p.gpu.download_constraints(m.copy())
    p.close()
    q = _split_pair(gpu_context, with_moving_kinematics(sb), sm, j)
    q.gpu.set_islands(isl, flags, idx)
    q.oracle.set_islands(isl, flags, idx)
    _run_exact(q, 3, 5)
    np.testing.assert_array_equal(q.gpu.get_islands()[0], q.oracle.get_islands()[0])
    q.close()


def test_pile_64k_both_prologues_equal(gpu_context):
    """The full pile: in-kernel (its default) and split prologues give the same
    bytes, and the default equals the oracle."""
    b, m, _ = scenes.pile_64k()
    gpu_context.set_settings(default_settings())
    out = {}
    for mode in (0, 1):
        sp = GpuSpace(gpu_context, b, m)
        sp.set_group_prologue(mode)
        for _ in range(3):
            sp.step(float(DT))
        launches = sp.last_step_launches()
        gb = sp.download_bodies()
        gm, _ = sp.download_constraints()
        out[mode] = (gb, gm, launches)
        sp.close()
    assert out[1][2] == out[0][2] + 2  # the refresh/body and the prestep launches
    for f in ("position", "orientation", "linear_velocity", "angular_velocity", "velocity_time_below_limit"):
        assert out[0][0][f].tobytes() == out[1][0][f].tobytes(), f
    for f in ("penetration_impulse", "position", "normal"):
        assert out[0][1]["contacts"][f].tobytes() == out[1][1]["contacts"][f].tobytes(), f
    assert out[0][1]["sliding_impulse"].tobytes() == out[1][1]["sliding_impulse"].tobytes()
    p = Pair(gpu_context, b, m)
    p.step(steps=3)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


def test_mode_checks_and_switching(gpu_context):
    b, m, _ = scenes.make_tower(300, seed=3)
    gpu_context.set_settings(default_settings())
    sp = GpuSpace(gpu_context, b, m)
    for bad in (-2, 2):
        with pytest.raises(N.BepuError):
            sp.set_group_prologue(bad)
    for _ in range(3):  # the kinematic ground's first steps add a launch of their own
        sp.step(float(DT))
    base = sp.last_step_launches()  # a small scene: in-kernel by default
    sp.set_group_prologue(1)
    sp.step(float(DT))
    assert sp.last_step_launches() == base + 2
    sp.set_group_prologue(-1)
    sp.step(float(DT))
    assert sp.last_step_launches() == base
    sp.close()


def test_chains_default_to_the_split_prologue(gpu_context):
    """Groups holding joints and at least 8,192 constraints take the split by
    default; the full chains scene then equals its in-kernel run bit for bit."""
    s = default_settings()
    s["iteration_limit"] = 15
    gpu_context.set_settings(s)
    b, m, j = scenes.chains_8k()
    out = {}
    for mode in (-1, 0):
        sp = GpuSpace(gpu_context, b, m, j)
        sp.set_group_prologue(mode)
        for _ in range(2):
            sp.step(float(DT))
        gb = sp.download_bodies()
        gm, gj = sp.download_constraints(joints=j.copy())
        out[mode] = (gb, gm, gj, sp.last_step_launches())
        sp.close()
    assert out[-1][3] == out[0][3] + 2
    for f in ("position", "orientation", "linear_velocity", "angular_velocity"):
        assert out[-1][0][f].tobytes() == out[0][0][f].tobytes(), f
    assert out[-1][2]["impulse"].tobytes() == out[0][2]["impulse"].tobytes()
    assert out[-1][1]["contacts"]["penetration_impulse"].tobytes() == \
        out[0][1]["contacts"]["penetration_impulse"].tobytes()
