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
