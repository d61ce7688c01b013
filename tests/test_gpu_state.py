"""The state-record calls (bepugpu_step_state, bepugpu_download_state) against
the whole-record calls: the same bits, with 64 bytes a body and a manifold
instead of whole records."""
import numpy as np
import pytest

from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, body_states, default_settings

from parity import DT

pytestmark = pytest.mark.gpu


def _same_bodies(state: np.ndarray, records: np.ndarray):
    for f in N.BODY_STATE_DTYPE.names:
        assert state[f].tobytes() == np.ascontiguousarray(records[f]).tobytes(), f


def _same_manifolds(state: np.ndarray, records: np.ndarray):
    count = records["contact_count"]
    np.testing.assert_array_equal(state["contact_count"], count)
    live = np.arange(4)[None, :] < count[:, None]
    ids = np.where(live, records["contacts"]["id"], 0)
    imp = np.where(live, records["contacts"]["penetration_impulse"], np.float32(0))
    assert state["contact_id"].tobytes() == ids.astype(np.int32).tobytes()
    assert state["penetration_impulse"].tobytes() == imp.astype(np.float32).tobytes()
    fimp = np.where(live, records["contacts"]["friction_impulse"], np.float32(0))
    assert state["friction_impulse"].tobytes() == fimp.astype(np.float32).tobytes()
    for f in ("sliding_impulse", "twist_impulse", "sliding_axis"):
        assert state[f].tobytes() == np.ascontiguousarray(records[f]).tobytes(), f
    assert not state["reserved"].any()


@pytest.mark.parametrize("mover", [False, True])
def test_step_state_equals_step_host(gpu_context, mover):
    gpu_context.set_settings(default_settings())
    b, m, _ = scenes.pile_1k(seed=5)
    if mover:  # a moving kinematic ground: the kinematic stages come from the state records
        b[0]["linear_velocity"] = (0.1, 0.0, 0.0)
        b[0]["angular_velocity"] = (0.0, 0.05, 0.0)
    whole = GpuSpace(gpu_context, b, m)
    state = GpuSpace(gpu_context, b, m)
    hb, hm = b.copy(), m.copy()
    sb = body_states(b)
    sm = np.zeros(len(m), N.MANIFOLD_STATE_DTYPE)
    for step in range(6):
        if step == 3:  # the host moves a body between steps
            hb["linear_velocity"][5] += np.float32(0.5)
            sb["linear_velocity"][5] = hb["linear_velocity"][5]
        whole.step_host(hb, hm, DT)
        state.step_state(sb, sm, DT)
        _same_bodies(sb, hb)
        _same_manifolds(sm, hm)
    whole.close()
    state.close()


def test_step_state_with_joints_equals_step(gpu_context):
    gpu_context.set_settings(default_settings())
    b, m, j = scenes.make_chain(chains=6, links=8, loose_bodies=10, seed=8,
                                region=np.array([12.0, 6.0, 12.0], np.float32))
    plain = GpuSpace(gpu_context, b, m, j)
    state = GpuSpace(gpu_context, b, m, j)
    sb = body_states(b)
    for _ in range(4):
        plain.step(DT)
        state.step_state(sb, None, DT)
    gpu_context.synchronize()
    _same_bodies(sb, plain.download_bodies(b.copy()))
    pm, pj = plain.download_constraints(m.copy(), j.copy())
    _, sj = state.download_constraints(m.copy(), j.copy())
    assert pj.tobytes() == sj.tobytes()
    sm = np.zeros(len(m), N.MANIFOLD_STATE_DTYPE)
    state.download_state(None, sm)
    _same_manifolds(sm, pm)
    plain.close()
    state.close()


def test_download_state_after_step_and_errors(gpu_context):
    gpu_context.set_settings(default_settings())
    b, m, _ = scenes.make_tower(300, seed=12)
    sp = GpuSpace(gpu_context, b, m)
    for _ in range(3):
        sp.step(DT)
    sb = np.zeros(len(b), N.BODY_STATE_DTYPE)
    sm = np.zeros(len(m), N.MANIFOLD_STATE_DTYPE)
    sp.download_state(sb, sm)
    _same_bodies(sb, sp.download_bodies(b.copy()))
    _same_manifolds(sm, sp.download_constraints(m.copy())[0])
    with pytest.raises(N.ArgumentException):
        sp.step_state(sb[:-1].copy(), None, DT)
    with pytest.raises(N.ArgumentException):
        sp.step_state(sb, sm[:-1].copy(), DT)
    with pytest.raises(N.ArgumentException):
        sp.step_state(sb, None, -1.0)
    with pytest.raises(N.ArgumentException):
        sp.download_state(sb[:-1].copy(), None)
    # nothing changed on the refused calls
    again = np.zeros(len(b), N.BODY_STATE_DTYPE)
    sp.download_state(again, None)
    assert again.tobytes() == sb.tobytes()
    sp.close()
