"""Simulation islands on the device against the oracle: islands falling
asleep in the round robin, sleeping islands skipped, a moving kinematic body
waking the islands it touches, on the island-group path, the colour-sweep
path and the persistent kernel, with joints and with the narrow phase; the
island flags and deactivation index bit for bit."""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, default_settings, islands_of

from island_records import sleepy_pile, with_moving_kinematics
from parity import DT, Pair

pytestmark = pytest.mark.gpu

GROUPS_ON = (1, 1024, 4096, 64, 0)
GROUPS_OFF = (0, 1024, 4096, 64, 0)
PATHS = [(GROUPS_ON, N.MODE_GRAPH), (GROUPS_OFF, N.MODE_GRAPH), (GROUPS_OFF, N.MODE_PERSISTENT)]


def _islands_equal(p):
    gf, gi = p.gpu.get_islands()
    of, oi = p.oracle.get_islands()
    np.testing.assert_array_equal(gf, of)
    assert gi == oi
    return gf


def _set_islands(p, isl, flags=None, idx=0):
    p.gpu.set_islands(isl, flags, idx)
    p.oracle.set_islands(isl, flags, idx)


@pytest.mark.parametrize("policy,mode", PATHS)
def test_pile_falls_asleep_in_the_round_robin(gpu_context, policy, mode):
    b, m, j = sleepy_pile(nx=16, ny=4, nz=16)
    p = Pair(gpu_context, b, m, j, group_policy=policy, mode=mode)
    _set_islands(p, islands_of(b, m, j))
    seen_asleep = False
    for chunk in range(13):
        p.step(steps=10)
        errs, exact = p.compare()
        assert exact, (chunk, errs)
        flags = _islands_equal(p)
        seen_asleep |= not np.all(flags & N.ISLAND_ACTIVE)
    assert seen_asleep and not np.any(flags & N.ISLAND_ACTIVE)
    p.close()


@pytest.mark.parametrize("ground_at", [0, 100])
@pytest.mark.parametrize("policy,mode", PATHS)
def test_moving_ground_wakes_the_pile(gpu_context, policy, mode, ground_at):
    b, m, j = sleepy_pile(nx=6, ny=4, nz=6, ground_at=ground_at)
    isl = islands_of(b, m, j)
    p = Pair(gpu_context, b, m, j, group_policy=policy, mode=mode)
    _set_islands(p, isl)
    p.step(steps=140)
    flags = _islands_equal(p)
    assert not np.any(flags & N.ISLAND_ACTIVE)
    sb = p.gpu.download_bodies(b.copy())
    sm, _ = p.gpu.download_constraints(m.copy())
    _, idx = p.gpu.get_islands()
    p.close()
    q = Pair(gpu_context, with_moving_kinematics(sb), sm, j, group_policy=policy, mode=mode)
    _set_islands(q, isl, flags, idx)
    for chunk in range(4):
        q.step(steps=5)
        errs, exact = q.compare()
        assert exact, (chunk, errs)
        flags = _islands_equal(q)
    assert np.all(flags & N.ISLAND_ACTIVE)
    q.close()


def test_sleeping_scene_skips_its_work(gpu_context):
    """Once every island sleeps the group launch returns at once: the step's
    bodies and impulses stay bit for bit, and it takes a fraction of an awake
    step's device time."""
    b, m, j = sleepy_pile(nx=16, ny=4, nz=16)
    gpu_context.set_settings(default_settings())
    sp = GpuSpace(gpu_context, b, m, j)
    sp.set_islands(islands_of(b, m, j))
    awake = []
    for _ in range(150):
        sp.step(float(DT))
        if len(awake) < 20:
            awake.append(sp.last_step_ms())
    flags, _ = sp.get_islands()
    assert not np.any(flags & N.ISLAND_ACTIVE)
    b1 = sp.download_bodies(b.copy())
    m1, _ = sp.download_constraints(m.copy())
    asleep = []
    for _ in range(20):
        sp.step(float(DT))
        asleep.append(sp.last_step_ms())
    b2 = sp.download_bodies(b.copy())
    m2, _ = sp.download_constraints(m.copy())
    for f in ("position", "orientation", "linear_velocity", "angular_velocity"):
        np.testing.assert_array_equal(b1[f], b2[f], err_msg=f)
    np.testing.assert_array_equal(m1["contacts"]["penetration_impulse"], m2["contacts"]["penetration_impulse"])
    assert np.median(asleep) < np.median(awake)
    sp.close()


@pytest.mark.parametrize("policy", [GROUPS_ON, GROUPS_OFF])
def test_chains_with_islands(gpu_context, policy):
    b, m, j = scenes.make_chain(chains=24, links=10, loose_bodies=80, seed=8,
                                region=np.array([30.0, 12.0, 30.0], np.float32))
    b = b.copy()
    b["activity"] &= ~np.uint32(N.BODY_ALWAYS_ACTIVE)
    s = default_settings()
    s["iteration_limit"] = 15
    p = Pair(gpu_context, b, m, j, settings=s, group_policy=policy)
    _set_islands(p, islands_of(b, m, j))
    for chunk in range(6):
        p.step(steps=25)
        errs, exact = p.compare()
        assert exact, (chunk, errs)
        _islands_equal(p)
    p.close()


def test_narrow_phase_pairs_with_islands(gpu_context):
    b, m, j, shapes = sleepy_pile(nx=6, ny=4, nz=6, collide=True)
    p = Pair(gpu_context, b, m, j, shapes=shapes)
    p.step(flags=N.STEP_ALL | N.STEP_COLLIDE)  # contacts first: the islands follow them
    gm, _ = p.gpu.download_constraints(m.copy())
    gb = p.gpu.download_bodies(b.copy())
    _set_islands(p, islands_of(gb, gm, j))
    for chunk in range(8):
        p.step(flags=N.STEP_ALL | N.STEP_COLLIDE, steps=20)
        errs, exact = p.compare()
        assert exact, (chunk, errs)
        flags = _islands_equal(p)
    assert not np.all(flags & N.ISLAND_ACTIVE)
    p.close()


def test_set_islands_checks(gpu_context):
    b, m, j = sleepy_pile(nx=3, ny=3, nz=3)
    gpu_context.set_settings(default_settings())
    sp = GpuSpace(gpu_context, b, m, j)
    isl = islands_of(b, m, j)
    cases = []
    bad = isl.copy()
    bad[0] = 0  # the kinematic ground in an island
    cases.append((bad, None, 0))
    bad = isl.copy()
    bad[1] = -1  # a dynamic body without one
    cases.append((bad, None, 0))
    bad = isl.copy()
    bad[bad == 1] = 0  # an island without members
    cases.append((bad, None, 0))
    bad = isl.copy()
    top = np.flatnonzero(isl == 0)[-1]
    bad[top] = isl.max() + 1  # a contact between two islands
    cases.append((bad, None, 0))
    cases.append((isl, None, isl.max() + 1))  # index outside the list
    cases.append((isl, np.full(isl.max() + 1, 4, np.uint32), 0))  # unknown flag bits
    for of, flags, idx in cases:
        with pytest.raises(N.BepuError):
            sp.set_islands(of, flags, idx)
    sp.set_islands(isl)
    assert len(sp.get_islands()[0]) == isl.max() + 1
    # new constraints clear the islands: the scene has none until they are set again
    sp.upload_constraints(m, j)
    with pytest.raises(N.BepuError):
        sp.get_islands()
    sp.island_count = 0
    assert len(sp.get_islands()[0]) == 0
    sp.close()


def _sleepy_towers(n, seed):
    out = []
    for i, k in enumerate(scenes.batch_body_counts(n, 8, 96, seed)):
        b, m, _ = scenes.make_tower(int(k), seed=seed * 1000 + i)
        b = b.copy()
        b["activity"] &= ~np.uint32(N.BODY_ALWAYS_ACTIVE)
        out.append((b, m))
    return out


def _island_spaces(ctx, pool):
    spaces = []
    for b, m in pool:
        sp = GpuSpace(ctx, b, m)
        sp.set_islands(islands_of(b, m))
        spaces.append(sp)
    return spaces


def _assert_same_spaces(ctx, a, b, pool):
    for sa, sb, (bb, mm) in zip(a, b, pool):
        x, y = sa.download_bodies(bb.copy()), sb.download_bodies(bb.copy())
        for f in ("position", "orientation", "linear_velocity", "angular_velocity", "velocity_time_below_limit"):
            np.testing.assert_array_equal(x[f], y[f], err_msg=f)
        np.testing.assert_array_equal(sa.download_constraints(mm.copy())[0]["contacts"]["penetration_impulse"],
                                      sb.download_constraints(mm.copy())[0]["contacts"]["penetration_impulse"])
        fa, ia = sa.get_islands()
        fb, ib = sb.get_islands()
        np.testing.assert_array_equal(fa, fb)
        assert ia == ib


def test_batched_island_scenes_step_as_alone(gpu_context):
    """Towers with islands through bepugpu_batch_step (the batched island stage,
    then the batched groups) equal the same towers stepped one at a time, until
    and after their islands sleep."""
    from bepuphysics1_gb300.solver import batch_step, last_call_stats
    gpu_context.set_settings(default_settings())
    pool = _sleepy_towers(24, 7)
    alone = _island_spaces(gpu_context, pool)
    batched = _island_spaces(gpu_context, pool)
    for rnd in range(30):
        for sp in alone:
            for _ in range(8):
                sp.step(float(DT))
        batch_step(gpu_context, batched, float(DT), 8)
        if rnd == 10:
            launches, _ = last_call_stats(gpu_context)
            assert launches > 0  # the island scenes took the batched launch
    _assert_same_spaces(gpu_context, alone, batched, pool)
    asleep = sum(int(np.count_nonzero((sp.get_islands()[0] & N.ISLAND_ACTIVE) == 0)) for sp in batched)
    assert asleep > 0
    for sp in alone + batched:
        sp.close()


def test_served_island_scenes_step_as_alone(gpu_context):
    from bepuphysics1_gb300.serve import Server
    gpu_context.set_settings(default_settings())
    pool = _sleepy_towers(16, 9)
    alone = _island_spaces(gpu_context, pool)
    served = _island_spaces(gpu_context, pool)
    srv = Server(gpu_context, dt=float(DT))
    for sp in served:
        srv.add(sp)
    for rnd in range(12):
        for sp in alone:
            for _ in range(16):
                sp.step(float(DT))
        for sp in served:
            while srv.submit(sp.id, 16, rnd) == N.QUEUE_FULL:
                pass
        srv.drain()
        while len(srv.poll()):
            pass
    for sp in served:
        srv.release(sp)
    srv.close()
    _assert_same_spaces(gpu_context, alone, served, pool)
    for sp in alone + served:
        sp.close()
