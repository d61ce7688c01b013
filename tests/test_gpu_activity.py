"""The activity state on the device: the deactivation candidacy update and the
stabilization boost of the force update (EntityBase.cs:926-936, on by default
as DeactivationManager.cs:60 leaves it), bit-exact against the oracle on every
path, and the kinematic bodies' time flag deciding their position update."""
import numpy as np
import pytest

from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, batch_step, default_settings

from parity import DT, Pair

pytestmark = pytest.mark.gpu

SWEEP = (0, 1024, 4096, 256, 0)
GROUPS = (1, 1024, 4096, 256, 0)


def _mixed_activity(b):
    """Half the dynamic bodies not always active (their candidacy times run),
    a third of them not stabilized."""
    b = b.copy()
    dyn = np.nonzero(b["is_dynamic"])[0]
    b["activity"][dyn[::2]] = 0
    b["activity"][dyn[1::3]] |= N.BODY_NO_STABILIZATION
    return b


@pytest.mark.parametrize("policy", ["sweep", "groups"])
def test_settled_pile_60_steps_stabilized(gpu_context, policy):
    """The settled 1,000-box pile: its slow bodies take the boost step after
    step; 60 steps bit-exact, activity fields included."""
    b, m, _ = scenes.pile_1k()
    b = _mixed_activity(b)
    p = Pair(gpu_context, b, m, group_policy=SWEEP if policy == "sweep" else GROUPS)
    for _ in range(6):
        p.step(steps=10)
        errs, exact = p.compare()
        assert exact, errs
    gb, ob = p.gpu.download_bodies(), p.oracle.get_bodies()
    for f in ("activity", "previous_velocity", "velocity_time_below_limit", "position", "orientation"):
        np.testing.assert_array_equal(gb[f], ob[f], err_msg=f)
    # the boost acted: bodies were slowing, and some non-always-active ones became candidates
    assert (gb["activity"] & N.BODY_SLOWING).any()
    assert (gb["activity"] & N.BODY_DEACTIVATION_CANDIDATE).any()
    p.close()


def test_boost_changes_the_step(gpu_context):
    """With the boost off the same pile steps differently (the test above is not vacuous)."""
    b, m, _ = scenes.pile_1k()
    s_off = default_settings()
    s_off["use_stabilization"] = 0
    p_on = Pair(gpu_context, b, m)
    p_on.step(steps=5)
    v_on = p_on.gpu.download_bodies()["linear_velocity"]
    p_on.close()
    p_off = Pair(gpu_context, b, m, settings=s_off)
    p_off.step(steps=5)
    errs, exact = p_off.compare()
    assert exact, errs
    v_off = p_off.gpu.download_bodies()["linear_velocity"]
    p_off.close()
    gpu_context.set_settings(default_settings())
    assert not np.array_equal(v_on, v_off)


def test_persistent_mode_stabilized(gpu_context):
    b, m, _ = scenes.pile_1k(seed=5)
    p = Pair(gpu_context, _mixed_activity(b), m, mode=N.MODE_PERSISTENT, group_policy=SWEEP)
    p.step(steps=20)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


@pytest.mark.parametrize("policy", ["sweep", "groups"])
def test_kinematic_flags_and_positions(gpu_context, policy):
    """Towers on a ground whose time flag starts at -1 (active for two more
    steps), plus a kinematic mover; the mover stops halfway.  Flags, poses and
    velocities bit-exact at every step."""
    b, m, _ = scenes.make_tower(300, seed=21)
    b = b.copy()
    kin = np.nonzero(b["is_dynamic"] == 0)[0]
    assert len(kin) >= 1
    b["velocity_time_below_limit"][kin] = -1.0
    b["orientation"][kin[0]] = (0.0, 0.0087265, 0.0, 0.99996192)  # turned slightly, so renormalising shows
    p = Pair(gpu_context, b, m, group_policy=SWEEP if policy == "sweep" else GROUPS)
    for step in range(6):
        p.step(steps=1)
        gb, ob = p.gpu.download_bodies(), p.oracle.get_bodies()
        for f in ("activity", "previous_velocity", "velocity_time_below_limit", "orientation", "position",
                  "linear_velocity"):
            np.testing.assert_array_equal(gb[f], ob[f], err_msg=f"{f} at step {step}")
    assert (gb["velocity_time_below_limit"][kin] == 1).all()  # settled: inactive
    p.close()


def test_kinematic_mover_stops(gpu_context):
    b, m, _ = scenes.make_tower(200, seed=22)
    b = b.copy()
    kin = int(np.nonzero(b["is_dynamic"] == 0)[0][0])
    b["linear_velocity"][kin] = (0.0, 0.0, 0.25)
    b["velocity_time_below_limit"][kin] = -1.0  # the velocity setter's Activate() (SimulationIslandMember.cs:262-266)
    sp = GpuSpace(gpu_context, b, m, group_policy=GROUPS)
    import oracle
    o = oracle.OracleSpace(default_settings(), b, m)
    o.set_list_order(sp.colouring()[1])
    for _ in range(3):
        sp.step(DT)
    o.step(DT, N.STEP_ALL, 3)
    gb = sp.download_bodies()
    gb["linear_velocity"][kin] = 0  # the mover stops; its flag stays as the step left it
    sp.update_bodies(gb)
    o2 = oracle.OracleSpace(default_settings(), gb, o.get_constraints()[0])
    o2.set_list_order(sp.colouring()[1])
    for _ in range(4):
        sp.step(DT)
    o2.step(DT, N.STEP_ALL, 4)
    gb, ob = sp.download_bodies(), o2.get_bodies()
    for f in ("position", "orientation", "linear_velocity", "velocity_time_below_limit", "activity"):
        np.testing.assert_array_equal(gb[f], ob[f], err_msg=f)
    assert gb["velocity_time_below_limit"][kin] == 1
    sp.close()
    o.close()
    o2.close()


def test_batched_towers_with_settling_grounds(gpu_context):
    """Tower scenes whose grounds start active join the batched launch once the
    grounds have settled; every call matches the oracle."""
    import oracle
    spaces, refs = [], []
    for i, n in enumerate((40, 90, 150)):
        b, m, _ = scenes.make_tower(n, seed=100 + i)
        b = b.copy()
        b["velocity_time_below_limit"][b["is_dynamic"] == 0] = -1.0
        sp = GpuSpace(gpu_context, b, m, group_policy=GROUPS)
        o = oracle.OracleSpace(default_settings(), b, m)
        o.set_list_order(sp.colouring()[1])
        spaces.append(sp)
        refs.append(o)
    for steps in (1, 1, 3, 4):
        batch_step(gpu_context, spaces, DT, steps)
        for sp, o in zip(spaces, refs):
            o.step(DT, N.STEP_ALL, steps)
            gb, ob = sp.download_bodies(), o.get_bodies()
            for f in ("linear_velocity", "angular_velocity", "position", "activity", "velocity_time_below_limit"):
                np.testing.assert_array_equal(gb[f], ob[f], err_msg=f)
    for sp, o in zip(spaces, refs):
        sp.close()
        o.close()


def test_update_bodies_carries_activity(gpu_context):
    """bepugpu_update_bodies takes the activity fields as state; the download returns them."""
    b, m, _ = scenes.pile_1k(seed=9)
    p = Pair(gpu_context, b, m)
    p.step(steps=2)
    gb = p.gpu.download_bodies()
    gb["activity"] ^= N.BODY_NO_STABILIZATION
    gb["velocity_time_below_limit"][5] = 0.75
    p.gpu.update_bodies(gb)
    np.testing.assert_array_equal(p.gpu.download_bodies(), gb)
    p.close()
