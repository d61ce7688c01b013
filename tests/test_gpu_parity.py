"""Parity of the device solver with the oracle (colour-order single-threaded
restatement), through the C ABI."""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, colour_list, default_settings

from parity import DT, LONG_TOL, STEP_TOL, Pair

pytestmark = pytest.mark.gpu


def test_colouring_bit_exact(gpu_context):
    for b, m, _ in (scenes.pile_1k(), scenes.make_tower(700, seed=3)):
        sp = GpuSpace(gpu_context, b, m)
        col, order, k = sp.colouring()
        col2, order2, k2 = oracle.colour(b, m)
        assert k == k2
        np.testing.assert_array_equal(col, col2)
        np.testing.assert_array_equal(order, order2)
        sp.close()


def test_pile_1k_every_step(gpu_context):
    b, m, _ = scenes.pile_1k()
    p = Pair(gpu_context, b, m)
    assert p.colours > 2
    for step in range(10):
        p.step()
        errs, exact = p.compare()
        for k, v in errs.items():
            assert v <= STEP_TOL, (step, k, v)
    p.close()


def test_pile_1k_sixty_steps(gpu_context):
    b, m, _ = scenes.pile_1k()
    p = Pair(gpu_context, b, m)
    p.step(steps=60)
    errs, exact = p.compare()
    for k, v in errs.items():
        assert v <= LONG_TOL, (k, v)
    # with -fmad=false and the reference's evaluation order the sequences are
    # the same floating-point computation
    assert exact, errs
    p.close()


def test_persistent_mode_equals_graph_mode(gpu_context):
    b, m, _ = scenes.pile_1k()
    g = GpuSpace(gpu_context, b, m)
    q = GpuSpace(gpu_context, b, m)
    q.set_mode(N.MODE_PERSISTENT)
    for _ in range(5):
        g.step(DT)
        q.step(DT)
    gpu_context.synchronize()
    gb, qb = g.download_bodies(), q.download_bodies()
    np.testing.assert_array_equal(gb["linear_velocity"], qb["linear_velocity"])
    np.testing.assert_array_equal(gb["angular_velocity"], qb["angular_velocity"])
    np.testing.assert_array_equal(gb["position"], qb["position"])
    gm, _ = g.download_constraints()
    qm, _ = q.download_constraints()
    np.testing.assert_array_equal(gm["contacts"]["penetration_impulse"], qm["contacts"]["penetration_impulse"])
    g.close()
    q.close()


def test_persistent_mode_parity(gpu_context):
    b, m, _ = scenes.pile_1k(seed=99)
    p = Pair(gpu_context, b, m, mode=N.MODE_PERSISTENT)
    p.step(steps=5)
    gpu_context.synchronize()
    errs, exact = p.compare()
    assert exact, errs
    p.close()


def test_pile_64k_full_size(gpu_context):
    b, m, _ = scenes.pile_64k()
    assert len(b) == 65537 and len(m) == 65536 and scenes.contact_count(m) == 262144
    p = Pair(gpu_context, b, m)
    for _ in range(3):
        p.step()
        errs, exact = p.compare()
        for k, v in errs.items():
            assert v <= STEP_TOL, (k, v)
    assert exact
    p.close()


def test_pile_64k_full_size_colour_sweeps(gpu_context):
    """The colour-sweep path (k_prestep / k_warm / k_solve, one launch per
    colour) on the whole 65,536-box pile, island groups off."""
    b, m, _ = scenes.pile_64k()
    p = Pair(gpu_context, b, m, group_policy=(0, 1024, 4096, 64, 0))
    for _ in range(2):
        p.step()
        errs, exact = p.compare()
        assert exact, errs
    assert p.gpu.last_step_launches() > 2 * p.colours  # swept, not grouped
    p.close()


def test_packed_pile_64k_one_island(gpu_context):
    """The 1.05 m packing of the 1,000-box pile scaled to 64 x 16 x 64: its
    columns touch, so the pile is one island too large for a group and the
    default policy runs it as colour sweeps."""
    b, m, _ = scenes.make_pile(nx=64, ny=16, nz=64, spacing=1.05, size_min=1.0, size_max=1.0, jitter=0.05,
                               friction_min=0.6, friction_max=0.6, seed=11)
    assert len(m) > 150000
    p = Pair(gpu_context, b, m)
    assert p.colours >= 8
    p.step()
    errs, exact = p.compare()
    assert exact, errs
    prof = p.gpu.last_step_launches()
    assert prof > p.colours
    p.close()


def test_towers(gpu_context):
    b, m, _ = scenes.make_tower(900, seed=11)
    p = Pair(gpu_context, b, m)
    p.step(steps=30)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


@pytest.mark.parametrize("flags", [N.STEP_FORCES, N.STEP_SOLVE, N.STEP_POSITIONS, N.STEP_REFRESH_CONTACTS,
                                   N.STEP_FORCES | N.STEP_SOLVE])
def test_single_stages(gpu_context, flags):
    b, m, _ = scenes.pile_1k(seed=5)
    b["linear_velocity"] = np.random.default_rng(1).normal(0, 0.5, (len(b), 3)).astype(np.float32)
    b["angular_velocity"] = np.random.default_rng(2).normal(0, 0.5, (len(b), 3)).astype(np.float32)
    b["linear_velocity"][0] = 0
    b["angular_velocity"][0] = 0
    p = Pair(gpu_context, b, m)
    p.step(flags=flags, steps=3)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


def test_bounciness_and_iteration_settings(gpu_context):
    b, m, _ = scenes.pile_1k(seed=7)
    m["bounciness"] = 0.5
    b["linear_velocity"][1:, 1] = -3.0
    s = default_settings()
    s["iteration_limit"] = 15
    s["minimum_iteration_count"] = 3
    s["maximum_iteration_count"] = 7
    p = Pair(gpu_context, b, m, settings=s)
    p.step(steps=4)
    errs, exact = p.compare()
    assert exact, errs
    p.close()
    gpu_context.set_settings(default_settings())


def test_null_entity_and_empty_manifolds(gpu_context):
    b, m, _ = scenes.pile_1k(seed=8)
    ground = m["body_a"] == 0
    m["body_a"][ground] = -1           # a static collidable that is not an entity
    m["contact_count"][::17] = 0       # manifolds that lost every contact
    m["flags"][::23] = N.MANIFOLD_ACTIVE  # collision rule NoSolver
    p = Pair(gpu_context, b, m)
    p.step(steps=5)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


def test_kinematic_mover(gpu_context):
    b, m, _ = scenes.pile_1k(seed=9)
    b[0]["linear_velocity"] = (0.1, 0.0, 0.0)   # a moving kinematic ground
    b[0]["angular_velocity"] = (0.0, 0.05, 0.0)
    p = Pair(gpu_context, b, m)
    p.step(steps=5)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


def test_empty_scene(gpu_context):
    b, m, _ = scenes.pile_1k()
    sp = GpuSpace(gpu_context, b, m[:0])
    sp.step(DT)
    out = sp.download_bodies()
    o = oracle.OracleSpace(default_settings(), b, m[:0])
    o.step(DT, N.STEP_ALL, 1)
    np.testing.assert_array_equal(out["position"], o.get_bodies()["position"])
    sp.close()


def test_errors_are_reported(gpu_context):
    b, m, _ = scenes.pile_1k()
    sp = GpuSpace(gpu_context, b, m)
    bad = m.copy()
    bad["contact_count"][3] = 5
    with pytest.raises(N.ArgumentException):
        sp.upload_constraints(bad)
    bad = m.copy()
    bad["body_b"][0] = len(b) + 1
    with pytest.raises(N.ArgumentException):
        sp.upload_constraints(bad)
    with pytest.raises(N.ArgumentException):
        sp.step(0.0)
    with pytest.raises(N.ArgumentException):
        sp.update_manifolds(m[:-1])
    with pytest.raises(N.ArgumentException):
        sp.upload_bodies(np.concatenate([b, b]))   # beyond capacity
    sp.close()
    with pytest.raises(N.ArgumentException):
        sp.id = 12345
        sp.step(DT)


def test_update_manifolds_round_trip(gpu_context):
    """Download -> update -> step equals stepping straight through (warm-start
    impulses and sliding axes survive the host round trip)."""
    b, m, _ = scenes.pile_1k(seed=4)
    a = GpuSpace(gpu_context, b, m)
    c = GpuSpace(gpu_context, b, m)
    for _ in range(3):
        a.step(DT)
        c.step(DT)
        cm, _ = c.download_constraints(m.copy())
        cb = c.download_bodies(b.copy())
        c.upload_bodies(cb)
        c.update_manifolds(cm)
    ab, cb = a.download_bodies(), c.download_bodies()
    np.testing.assert_array_equal(ab["linear_velocity"], cb["linear_velocity"])
    a.close()
    c.close()


def test_manifold_records_roundtrip(gpu_context):
    """Downloading right after an upload gives back the uploaded records (whole
    records are rebuilt on the device)."""
    gpu_context.set_settings(default_settings())
    b, m, _ = scenes.pile_1k()
    m = m.copy()
    rng = np.random.default_rng(2)
    live = np.arange(4)[None, :] < m["contact_count"][:, None]
    m["contacts"]["penetration_impulse"] = np.where(live, rng.uniform(0, 1, live.shape), 0).astype(np.float32)
    m["sliding_impulse"] = rng.normal(size=m["sliding_impulse"].shape).astype(np.float32)
    m["twist_impulse"] = rng.normal(size=m["twist_impulse"].shape).astype(np.float32)
    m["contact_order"] = 0
    sp = GpuSpace(gpu_context, b, m)
    back, _ = sp.download_constraints(np.zeros_like(m))
    assert back.tobytes() == m.tobytes()
    sp.close()


def test_update_bodies_and_manifolds_per_step(gpu_context):
    """The per-step update calls (device-checked) give the same bits as full
    uploads, refuse records that change more than their state, and a kinematic
    body set moving by an update is integrated."""
    gpu_context.set_settings(default_settings())
    b, m, _ = scenes.pile_1k()
    full = GpuSpace(gpu_context, b, m)
    fast = GpuSpace(gpu_context, b, m)
    hb, hm = b.copy(), m.copy()
    for _ in range(3):
        full.upload_bodies(hb)
        full.update_manifolds(hm)
        fast.update_bodies(hb)
        fast.update_manifolds(hm)
        full.step(DT)
        fast.step(DT)
        hb = full.download_bodies(hb.copy())
        hm = full.download_constraints(hm.copy())[0]
        fb = fast.download_bodies(hb.copy())
        fm = fast.download_constraints(hm.copy())[0]
        assert fb.tobytes() == hb.tobytes() and fm.tobytes() == hm.tobytes()
    bad = hb.copy()
    bad["inverse_mass"][5] *= 2
    with pytest.raises(N.ArgumentException):
        fast.update_bodies(bad)
    bad = hm.copy()
    bad["body_b"][7] = bad["body_a"][7]
    with pytest.raises(N.ArgumentException):
        fast.update_manifolds(bad)
    # the ground (kinematic, body 0) starts moving: integrated like the oracle does
    moving = hb.copy()
    moving["linear_velocity"][0] = (0.0, 0.5, 0.0)
    fast.update_bodies(moving)
    fast.step(DT)
    ref = oracle.OracleSpace(default_settings(), moving, hm)
    ref.set_list_order(fast.colouring()[1])
    ref.step(DT, N.STEP_ALL, 1)
    got = fast.download_bodies(moving.copy())
    assert np.array_equal(got["position"], ref.get_bodies()["position"])
    full.close()
    fast.close()


def test_step_host_equals_separate_calls(gpu_context):
    """bepugpu_step_host gives the bits of update, step and download done
    separately, refuses a bad record with nothing changed, and takes no scene
    with joints."""
    gpu_context.set_settings(default_settings())
    b, m, _ = scenes.pile_1k()
    calls = GpuSpace(gpu_context, b, m)
    one = GpuSpace(gpu_context, b, m)
    hb, hm = b.copy(), m.copy()
    ob, om = b.copy(), m.copy()
    for _ in range(4):
        calls.update_bodies(hb)
        calls.update_manifolds(hm)
        calls.step(DT)
        hb = calls.download_bodies(hb)
        hm = calls.download_constraints(hm)[0]
        one.step_host(ob, om, DT)
        assert ob.tobytes() == hb.tobytes() and om.tobytes() == hm.tobytes()
    before = one.download_bodies(ob.copy())
    bad = ob.copy()
    bad["inverse_mass"][3] *= 2
    with pytest.raises(N.ArgumentException):
        one.step_host(bad, om.copy(), DT)
    badm = om.copy()
    badm["contact_count"][2] = 7
    with pytest.raises(N.ArgumentException):
        one.step_host(ob.copy(), badm, DT)
    assert one.download_bodies(ob.copy()).tobytes() == before.tobytes()
    calls.close()
    one.close()
    cb, cm, cj = scenes.make_chain(chains=2, links=4, loose_bodies=2, seed=4,
                                   region=np.array([6.0, 4.0, 6.0], np.float32))
    sj = GpuSpace(gpu_context, cb, cm, cj)
    with pytest.raises(N.InvalidOperationException):
        sj.step_host(cb.copy(), cm.copy(), DT)
    sj.close()


def test_check_finite_and_bounded_wait(gpu_context):
    """NaN state is reported as NAN_DETECTED with the body's index; a device
    wait on a flag nothing sets gives up with TIMEOUT and the context keeps
    working."""
    gpu_context.set_settings(default_settings())
    b, m, _ = scenes.pile_1k()
    sp = GpuSpace(gpu_context, b, m)
    assert sp.check_finite() == -1
    bad = b.copy()
    bad["linear_velocity"][17] = (np.nan, 0, 0)
    bad["angular_velocity"][40] = (0, np.inf, 0)
    sp.upload_bodies(bad)
    with pytest.raises(N.BepuError) as err:
        sp.check_finite()
    assert err.value.status == N.NAN_DETECTED and "body 17" in str(err.value)
    st = gpu_context.lib.bepugpu_probe_bounded_wait(gpu_context.handle, 1000)
    assert st == N.TIMEOUT
    sp.upload_bodies(b)
    sp.step(DT)
    assert sp.check_finite() == -1
    sp.close()
