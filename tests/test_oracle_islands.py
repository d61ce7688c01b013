"""The oracle's simulation islands: DeactivationManager.Update over a given
island list (DeactivationManagement/DeactivationManager.cs:216-336,
SimulationIsland.cs:94-118, SimulationIslandMember.cs:53-164) and the stages
that skip inactive bodies and constraints.

The reference has no golden vectors for deactivation; these tests pin the
restatement to the rules as the reference writes them: the round robin's
member budget and island count, TryToDeactivate's all-candidates test and its
one-attempt allowDeactivation reset, a moving kinematic body waking the islands
it touches from its own turn in the member loop, and sleeping islands frozen
with their constraints' impulses kept.
"""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300.solver import default_settings, islands_of

from island_records import sleepy_pile, with_moving_kinematics

DT = np.float32(1 / 60)
AWAKE = N.ISLAND_ACTIVE | N.ISLAND_ALLOW_DEACTIVATION


def _space(b, m, j=None, **settings):
    s = default_settings()
    for k, v in settings.items():
        s[k] = v
    o = oracle.OracleSpace(s, b, m, j)
    return o


def test_islands_of_columns():
    b, m, j = sleepy_pile(nx=4, ny=3, nz=4)
    isl = islands_of(b, m, j)
    assert isl[0] == -1  # the kinematic ground
    assert isl.max() + 1 == 16
    np.testing.assert_array_equal(np.bincount(isl[isl >= 0]), np.full(16, 3))


def test_round_robin_budget_and_progressive_sleep():
    """Every step DeactivateObjects looks at islands until their members add up
    to the budget (DeactivationManager.cs:318-335): 25 four-box columns per step
    at the default 100, so the index advances by 25 and at most 25 islands fall
    asleep in one step."""
    b, m, j = sleepy_pile(nx=16, ny=4, nz=16)
    o = _space(b, m, j)
    isl = islands_of(b, m, j)
    o.set_islands(isl)
    asleep_before, idx_before = 0, 0
    slept_any = False
    for step in range(130):
        o.step(DT)
        flags, idx = o.get_islands()
        assert idx == (idx_before + 25) % 256
        asleep = int(np.count_nonzero((flags & N.ISLAND_ACTIVE) == 0))
        assert 0 <= asleep - asleep_before <= 25
        slept_any |= asleep > 0
        asleep_before, idx_before = asleep, idx
    assert asleep_before == 256 and slept_any
    # the budget counts members, not islands
    o2 = _space(b, m, j, maximum_deactivation_attempts_per_frame=7)
    o2.set_islands(isl)
    o2.step(DT)
    assert o2.get_islands()[1] == 2  # islands 1 and 2: 4 + 4 members >= 7


def test_sleeping_islands_are_frozen():
    b, m, j = sleepy_pile(nx=6, ny=4, nz=6)
    o = _space(b, m, j)
    o.set_islands(islands_of(b, m, j))
    o.step(DT, steps=140)
    flags, _ = o.get_islands()
    assert not np.any(flags & N.ISLAND_ACTIVE)
    b1, (m1, _) = o.get_bodies(), o.get_constraints()
    o.step(DT, steps=20)
    b2, (m2, _) = o.get_bodies(), o.get_constraints()
    for f in ("position", "orientation", "linear_velocity", "angular_velocity", "previous_velocity"):
        np.testing.assert_array_equal(b1[f], b2[f], err_msg=f)
    np.testing.assert_array_equal(m1["contacts"]["penetration_impulse"], m2["contacts"]["penetration_impulse"])
    # without islands the same bodies keep moving
    o3 = _space(b1, m1, j)
    o3.step(DT, steps=5)
    assert not np.array_equal(o3.get_bodies()["position"], b1["position"])


@pytest.mark.parametrize("ground_at", [0, 40, 144])
def test_moving_kinematic_wakes_its_islands(ground_at):
    """A sleeping pile on a ground that starts moving: at the ground's turn in
    the member loop every island it touches wakes and loses one deactivation
    attempt (SimulationIslandMember.cs:135-159); members before the ground in
    the list are not updated as active in that step, members after it are."""
    b, m, j = sleepy_pile(nx=6, ny=4, nz=6, ground_at=ground_at)
    isl = islands_of(b, m, j)
    o = _space(b, m, j)
    o.set_islands(isl)
    o.step(DT, steps=140)
    flags, idx = o.get_islands()
    assert not np.any(flags & N.ISLAND_ACTIVE)
    sb = o.get_bodies()
    sm, _ = o.get_constraints()
    moving = with_moving_kinematics(sb)
    o2 = _space(moving, sm, j)
    o2.set_islands(isl, flags, idx)
    o2.step(DT)
    f2, idx2 = o2.get_islands()
    assert np.all(f2 & N.ISLAND_ACTIVE)
    # the islands DeactivateObjects looked at this step got their attempt back
    looked = [(idx + 1 + k) % len(f2) for k in range(25)]
    allowed = (f2 & N.ISLAND_ALLOW_DEACTIVATION) != 0
    assert allowed[looked].all() and not np.delete(allowed, looked).any()
    # the candidacy update ran for the members after the ground only
    nb = o2.get_bodies()
    dyn = np.flatnonzero(sb["is_dynamic"] == 1)
    changed = nb["velocity_time_below_limit"][dyn] != sb["velocity_time_below_limit"][dyn]
    np.testing.assert_array_equal(changed, dyn > ground_at)


def test_set_islands_checks_the_partition():
    b, m, j = sleepy_pile(nx=3, ny=3, nz=3)
    isl = islands_of(b, m, j)
    o = _space(b, m, j)
    bad = isl.copy()
    bad[0] = 0  # the kinematic ground in an island
    with pytest.raises(ValueError):
        o.set_islands(bad)
    bad = isl.copy()
    bad[bad == 1] = 0  # island 1 left without a member
    with pytest.raises(ValueError):
        o.set_islands(bad)
    merged = bad.copy()
    merged[merged > 1] -= 1  # two columns as one island: a partition the host may keep
    o.set_islands(merged)
    assert o.get_islands()[0].shape == (isl.max(),)


def test_set_islands_refuses_split_connections():
    b, m, j = sleepy_pile(nx=3, ny=3, nz=3)
    isl = islands_of(b, m, j)
    o = _space(b, m, j)
    bad = isl.copy()
    first = np.flatnonzero(isl == 0)
    bad[first[-1]] = isl.max() + 1  # a column's top box alone: its contact spans two islands
    with pytest.raises(ValueError):
        o.set_islands(bad)
    empty = np.full(isl.max() + 2, AWAKE, np.uint32)
    with pytest.raises(ValueError):
        o.set_islands(isl, empty)
