"""A dropped pile settled on the device -- broad phase, pair records, narrow
phase and solver each step -- against the oracle running the same loop with
its own broad phase: the pair sets equal every step, and bodies, contacts
and impulses bit for bit."""
import numpy as np
import pytest

import oracle
from oracle.broad_phase import overlapping_pairs
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.pairs import PairRecords, settle
from bepuphysics1_gb300.solver import GpuSpace, default_settings

from parity import compare

pytestmark = pytest.mark.gpu

DT = np.float32(1 / 60)
FLAGS = N.STEP_ALL | N.STEP_COLLIDE


@pytest.mark.parametrize("policy", [None, (0, 1024, 4096, 64, 0)])
def test_dropped_pile_settles_like_the_oracle(gpu_context, policy):
    b, shapes, fr = scenes.dropped_pile(nx=5, ny=4, nz=5, seed=77)
    s = default_settings()
    gpu_context.set_settings(s)
    nb = len(b)
    sp = GpuSpace(gpu_context, b, None, capacity=(nb, 16 * nb, 0), group_policy=policy, shapes=shapes)
    g_rec, o_rec = PairRecords(fr, shapes), PairRecords(fr, shapes)
    o = None
    o_bodies = b
    changes = 0
    for step in range(140):
        pairs = sp.broad_phase(float(DT))
        np.testing.assert_array_equal(pairs, overlapping_pairs(o_bodies, shapes, DT), err_msg=str(step))
        g_cur = sp.download_constraints(g_rec.manifolds.copy())[0] if len(g_rec.manifolds) else None
        o_cur = o.get_constraints()[0] if o is not None else None
        changed = g_rec.update(pairs, g_cur)
        assert o_rec.update(pairs, o_cur) == changed
        if changed or o is None:
            changes += 1
            sp.upload_constraints(g_rec.manifolds)
            o = oracle.OracleSpace(s, o_bodies, o_rec.manifolds, shapes=shapes)
            o.set_list_order(sp.colouring()[1])
            o.set_order_mode(oracle.ORDER_IDENTITY)
        sp.step(float(DT), FLAGS)
        o.step(DT, FLAGS)
        o_bodies = o.get_bodies()
        if step % 10 == 9 or changed:
            gb = sp.download_bodies(b.copy())
            gm, _ = sp.download_constraints(g_rec.manifolds.copy())
            om, _ = o.get_constraints()
            errs, exact = compare(gb, gm, o_bodies, om)
            assert exact, (step, errs)
    assert changes > 3
    sp.close()


def test_settle_helper_runs_the_loop(gpu_context):
    b, shapes, fr = scenes.dropped_pile(nx=4, ny=3, nz=4, seed=5)
    gpu_context.set_settings(default_settings())
    nb = len(b)
    sp = GpuSpace(gpu_context, b, None, capacity=(nb, 16 * nb, 0), shapes=shapes)
    records = PairRecords(fr, shapes)
    changes = settle(sp, records, float(DT), 120)
    assert changes > 3
    gb = sp.download_bodies(b.copy())
    gm, _ = sp.download_constraints(records.manifolds.copy())
    dyn = gb["is_dynamic"] == 1
    assert float(np.abs(gb["linear_velocity"][dyn]).max()) < 1.0
    assert int(gm["contact_count"].sum()) >= 4 * int(dyn.sum())
    sp.close()


def _device_space(ctx, b, shapes, fr, policy=None):
    nb = len(b)
    sp = GpuSpace(ctx, b, None, capacity=(nb, 16 * nb, 0), group_policy=policy, shapes=shapes)
    sp.set_materials(np.stack([fr, fr, np.zeros_like(fr)], 1))
    return sp


@pytest.mark.parametrize("seed", [77, 78])
def test_device_pair_updates_equal_the_host_loop(gpu_context, seed):
    """bepugpu_update_pairs against the host loop (download, PairRecords diff,
    upload_constraints): the same records, colouring and steps bit for bit."""
    b, shapes, fr = scenes.dropped_pile(nx=5, ny=4, nz=5, seed=seed)
    gpu_context.set_settings(default_settings())
    dev = _device_space(gpu_context, b, shapes, fr)
    host = GpuSpace(gpu_context, b, None, capacity=(len(b), 16 * len(b), 0), shapes=shapes)
    rec = PairRecords(fr, shapes)
    for step in range(120):
        n = dev.update_pairs(float(DT))
        pairs = host.broad_phase(float(DT))
        cur = host.download_constraints(rec.manifolds.copy())[0] if len(rec.manifolds) else None
        if rec.update(pairs, cur) or step == 0:
            host.upload_constraints(rec.manifolds)
        assert n == len(rec.manifolds), step
        if step % 15 == 0:
            dcol, dord, dk = dev.colouring()
            hcol, hord, hk = host.colouring()
            np.testing.assert_array_equal(dcol, hcol, err_msg=str(step))
            np.testing.assert_array_equal(dord, hord, err_msg=str(step))
        dev.step(float(DT), FLAGS)
        host.step(float(DT), FLAGS)
        if step % 10 == 9:
            db = dev.download_bodies(b.copy())
            hb = host.download_bodies(b.copy())
            dm, _ = dev.download_constraints(rec.manifolds.copy())
            hm, _ = host.download_constraints(rec.manifolds.copy())
            for f in ("position", "orientation", "linear_velocity", "angular_velocity"):
                np.testing.assert_array_equal(db[f], hb[f], err_msg=f"{step} {f}")
            np.testing.assert_array_equal(dm, hm, err_msg=str(step))
    dev.close()
    host.close()


def test_device_colouring_equals_the_host_colouring(gpu_context):
    """The device colouring of a big settled heap equals bepugpu_colour_list on
    the same records (greedy in list order, conflicts through dynamic bodies)."""
    from bepuphysics1_gb300.solver import colour_list
    b, shapes, fr = scenes.dropped_pile(nx=12, ny=8, nz=12, seed=3)
    gpu_context.set_settings(default_settings())
    dev = _device_space(gpu_context, b, shapes, fr)
    for _ in range(150):
        dev.update_pairs(float(DT))
        dev.step(float(DT), FLAGS)
    dev.update_pairs(float(DT))
    m, _ = dev.download_constraints()
    bb = dev.download_bodies(b.copy())
    col, order, k = dev.colouring()
    hcol, hord, hk = colour_list(bb, m)
    np.testing.assert_array_equal(col, hcol)
    np.testing.assert_array_equal(order, hord)
    assert k == hk and k > 4
    dev.close()


def test_update_pairs_checks(gpu_context):
    b, shapes, fr = scenes.dropped_pile(nx=3, ny=2, nz=3, seed=9)
    gpu_context.set_settings(default_settings())
    sp = GpuSpace(gpu_context, b, None, capacity=(len(b), 2, 0), shapes=shapes)
    with pytest.raises(N.BepuError):  # no materials yet
        sp.update_pairs(float(DT))
    sp.set_materials(np.ones((len(b), 3), np.float32))
    for _ in range(30):  # with no manifolds the bottom layer sinks into the ground: nine pairs, capacity 2
        sp.step(float(DT), N.STEP_ALL)
    with pytest.raises(N.BepuError):
        sp.update_pairs(float(DT))
    sp.close()
