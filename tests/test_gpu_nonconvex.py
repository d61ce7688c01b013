"""NonConvexContactManifoldConstraint on the device: per-contact friction
children (ContactFrictionConstraint) after the penetration children, checked
bit for bit against the oracle's colour-order run -- frozen four-contact
manifolds with the refresher removing contacts, the scene source's sphere
pairs, narrow-phase sphere pairs, every solve path, and the record and
state round trips."""
import numpy as np
import pytest

from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, body_states, default_settings

from parity import DT, Pair
from test_gpu_collide import _all_pairs, _jumble

pytestmark = pytest.mark.gpu


def _nonconvex(m, every=1):
    m = m.copy()
    m["flags"][::every] |= N.MANIFOLD_NONCONVEX
    return m


def _assert_exact(p, steps, every_step=True):
    for s in range(steps):
        p.step()
        if every_step or s == steps - 1:
            errs, exact = p.compare()
            assert exact, (s, errs)
            gm, _ = p.gpu.download_constraints()
            om, _ = p.oracle.get_constraints()
            for f in ("friction_impulse", "friction_direction"):
                assert gm["contacts"][f].tobytes() == om["contacts"][f].tobytes(), (s, f)


@pytest.mark.parametrize("policy", [None, (0, 1024, 4096, 64, 0)])
def test_pile_all_nonconvex(gpu_context, policy):
    """Four-contact frozen manifolds, all nonconvex: the refresher drops
    contacts (their friction children go with them), island groups keep such
    manifolds' lanes in global memory."""
    b, m, _ = scenes.pile_1k(seed=4)
    p = Pair(gpu_context, b, _nonconvex(m), group_policy=policy)
    _assert_exact(p, 12)
    p.close()


def test_pile_mixed_sixty_steps_and_persistent(gpu_context):
    b, m, _ = scenes.pile_1k(seed=6)
    m = _nonconvex(m, every=3)
    p = Pair(gpu_context, b, m)
    _assert_exact(p, 60, every_step=False)
    p.close()
    q = Pair(gpu_context, b, m, mode=N.MODE_PERSISTENT)
    _assert_exact(q, 10, every_step=False)
    q.close()


def test_scene_source_sphere_pairs_are_nonconvex(gpu_context):
    """Towers of boxes and spheres: the scene source flags sphere-sphere and
    box-sphere pairs nonconvex, as the reference's pair handlers build them."""
    b, m, _ = scenes.make_tower(600, seed=14, sphere_fraction=0.5)
    nonconvex = (m["flags"] & N.MANIFOLD_NONCONVEX) != 0
    assert nonconvex.any() and (~nonconvex).any()
    p = Pair(gpu_context, b, m)
    _assert_exact(p, 30, every_step=False)
    p.close()


def test_narrow_phase_sphere_pairs(gpu_context):
    """GENERATED sphere-sphere and box-sphere pairs, nonconvex as in the
    reference, beside box-box pairs, both convex and (for coverage of the
    contact moves) nonconvex."""
    b, m, sh = _jumble(seed=9, n=200, sphere_every=3)
    sphere = sh["type"] == N.SHAPE_SPHERE
    with_sphere = sphere[m["body_a"]] | sphere[m["body_b"]]
    m["flags"][with_sphere] |= N.MANIFOLD_NONCONVEX
    boxbox = np.flatnonzero(~with_sphere)
    m["flags"][boxbox[::2]] |= N.MANIFOLD_NONCONVEX
    p = Pair(gpu_context, b, m, shapes=sh)
    _assert_exact(p, 20)
    p.close()


def test_records_round_trip_resumes_bit_for_bit(gpu_context):
    """Whole records carry each contact's friction impulse and direction: a
    scene rebuilt from downloaded records continues exactly."""
    gpu_context.set_settings(default_settings())
    b, m, _ = scenes.pile_1k(seed=8)
    m = _nonconvex(m, every=2)
    whole = GpuSpace(gpu_context, b, m)
    for _ in range(5):
        whole.step(DT)
    rb = whole.download_bodies(b.copy())
    rm, _ = whole.download_constraints(m.copy())
    assert (rm["contacts"]["friction_impulse"] != 0).any()
    resumed = GpuSpace(gpu_context, rb, rm)
    for _ in range(5):
        whole.step(DT)
        resumed.step(DT)
    gpu_context.synchronize()
    assert whole.download_bodies(b.copy()).tobytes() == resumed.download_bodies(b.copy()).tobytes()
    assert whole.download_constraints(m.copy())[0].tobytes() == resumed.download_constraints(m.copy())[0].tobytes()
    whole.close()
    resumed.close()


def test_state_records_carry_contact_friction(gpu_context):
    gpu_context.set_settings(default_settings())
    b, m, _ = scenes.make_tower(400, seed=15, sphere_fraction=0.5)
    sp = GpuSpace(gpu_context, b, m)
    sb = body_states(b)
    sm = np.zeros(len(m), N.MANIFOLD_STATE_DTYPE)
    for _ in range(4):
        sp.step_state(sb, sm, DT)
    rm, _ = sp.download_constraints(m.copy())
    live = np.arange(4)[None, :] < rm["contact_count"][:, None]
    want = np.where(live, rm["contacts"]["friction_impulse"], np.float32(0))
    assert sm["friction_impulse"].tobytes() == want.astype(np.float32).tobytes()
    assert (sm["friction_impulse"] != 0).any()
    sp.close()


def test_nonconvex_flag_cannot_change_without_upload(gpu_context):
    b, m, _ = scenes.pile_1k(seed=2)
    sp = GpuSpace(gpu_context, b, m)
    bad = m.copy()
    bad["flags"][7] |= N.MANIFOLD_NONCONVEX
    with pytest.raises(N.ArgumentException):
        sp.update_manifolds(bad)
    sp.close()
