"""The device broad phase (bepugpu_broad_phase) against the oracle's
brute-force restatement of the reference's bounding boxes and overlap test:
the same pair set, bit for bit in the boxes that decide it."""
import numpy as np
import pytest

from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, default_settings
from oracle import broad_phase as obp

from parity import DT
from test_gpu_collide import _jumble

pytestmark = pytest.mark.gpu


def _moving(b, seed, scale=3.0):
    b = b.copy()
    rng = np.random.default_rng(seed)
    dyn = b["is_dynamic"] != 0
    b["linear_velocity"][dyn] = rng.uniform(-scale, scale, (int(dyn.sum()), 3)).astype(np.float32)
    return b


@pytest.mark.parametrize("dt", [0.0, float(DT), 0.25])
def test_jumble_pairs_equal_brute_force(gpu_context, dt):
    """Turned boxes and spheres with velocities: rotated boxes' extreme points,
    the velocity expansion on each side, kinematic-kinematic exclusion."""
    b, m, sh = _jumble(seed=5, n=240, sphere_every=3)
    b = _moving(b, 5)
    sp = GpuSpace(gpu_context, b, m, shapes=sh)
    got = sp.broad_phase(dt)
    want = obp.overlapping_pairs(b, sh, dt)
    assert len(want) > len(b)
    np.testing.assert_array_equal(got, want)
    sp.close()


def test_after_steps_and_with_unshaped_and_kinematic_bodies(gpu_context):
    """The boxes follow the device state after steps; bodies of shape NONE
    and pairs of kinematic bodies are left out."""
    gpu_context.set_settings(default_settings())
    b, m, _, sh = scenes.make_tower(900, seed=6, sphere_fraction=0.4, narrow_phase=1)
    sh = sh.copy()
    sh["type"][5:40:3] = N.SHAPE_NONE
    sh["size"][5:40:3] = 0
    b = b.copy()
    b["is_dynamic"][10:30:4] = 0  # some kinematic bodies beside the ground
    shaped = sh["type"] != N.SHAPE_NONE
    m = m[shaped[m["body_a"]] & shaped[m["body_b"]]]  # the narrow phase needs both shapes
    sp = GpuSpace(gpu_context, b, m, shapes=sh)
    for _ in range(5):
        sp.step(DT)
    now = sp.download_bodies(b.copy())
    got = sp.broad_phase(DT)
    np.testing.assert_array_equal(got, obp.overlapping_pairs(now, sh, DT))
    dyn = now["is_dynamic"] != 0
    assert (dyn[got[:, 0]] | dyn[got[:, 1]]).all()
    assert (sh["type"][got.ravel()] != N.SHAPE_NONE).all()
    sp.close()


def test_pile_8k_and_truncated_output(gpu_context):
    """An 8,192-box pile (four sort tiles): the full set, then a call with room
    for fewer pairs writes the ascending prefix and reports the full count."""
    b, m, _, sh = scenes.make_pile(nx=32, ny=8, nz=32, narrow_phase=1, seed=31)
    b = _moving(b, 31, scale=1.0)
    sp = GpuSpace(gpu_context, b, m, shapes=sh)
    want = obp.overlapping_pairs(b, sh, DT)
    got = sp.broad_phase(DT)
    np.testing.assert_array_equal(got, want)
    import ctypes
    cap = len(want) // 3
    out = np.zeros((cap, 2), np.int32)
    n = ctypes.c_uint32()
    gpu_context.check(gpu_context.lib.bepugpu_broad_phase(gpu_context.handle, sp.id, float(DT), N.ptr(out), cap,
                                                          ctypes.byref(n)))
    assert n.value == len(want)
    np.testing.assert_array_equal(out, want[:cap])
    sp.close()


def test_pile_64k_full_size_properties(gpu_context):
    """The 65,536-box pile: every reported pair overlaps, the list is sorted
    and unique, and each manifold's pair of the narrow-phase scene is found."""
    b, m, _, sh = scenes.make_pile(nx=64, ny=16, nz=64, narrow_phase=1, seed=1)
    sp = GpuSpace(gpu_context, b, m, shapes=sh)
    got = sp.broad_phase(DT)
    lo, hi = obp.bounding_boxes(b, sh, DT)
    a, c = got[:, 0], got[:, 1]
    assert (a < c).all()
    assert not ((lo[c] > hi[a]).any(axis=1) | (lo[a] > hi[c]).any(axis=1)).any()
    keys = a.astype(np.int64) * len(b) + c
    assert (np.diff(keys) > 0).all()
    # every candidate pair of the narrow-phase scene whose boxes overlap is found
    ma, mb = np.minimum(m["body_a"], m["body_b"]), np.maximum(m["body_a"], m["body_b"])
    overlap = ~((lo[mb] > hi[ma]).any(axis=1) | (lo[ma] > hi[mb]).any(axis=1))
    assert overlap.sum() > len(b)
    mk = ma.astype(np.int64) * len(b) + mb
    assert np.isin(mk[overlap], keys).all()
    sp.close()


def _line_of_boxes(n, spacing, half, wide_every=0, wide_half=40.0, seed=0):
    rng = np.random.default_rng(seed)
    b = np.zeros(n, N.BODY_DTYPE)
    b["orientation"] = (0, 0, 0, 1)
    b["is_dynamic"] = 1
    b["inverse_mass"] = 1
    b["local_inverse_inertia"] = (1, 0, 0, 0, 1, 0, 0, 0, 1)
    b["position"][:, 0] = np.arange(n, dtype=np.float32) * np.float32(spacing)
    b["position"][:, 1:] = rng.uniform(-0.2, 0.2, (n, 2)).astype(np.float32)
    sh = np.zeros(n, N.SHAPE_DTYPE)
    sh["type"] = N.SHAPE_BOX
    sh["size"] = half
    if wide_every:
        sh["size"][::wide_every, 0] = wide_half  # long boxes across many cells
    return b, sh


def test_grid_wraps_and_wide_bodies(gpu_context):
    """A line of boxes far longer than 1,024 cells (the cell codes wrap, so
    far-apart cells share a code) with long boxes among them (wide bodies,
    tested against all, pairs of two wide bodies reported once)."""
    b, sh = _line_of_boxes(6000, 1.9, 1.0, wide_every=31)
    m = np.zeros(0, N.MANIFOLD_DTYPE)
    sp = GpuSpace(gpu_context, b, m, shapes=sh)
    for dt in (0.0, float(DT)):
        got = sp.broad_phase(dt)
        want = obp.overlapping_pairs(b, sh, dt)
        np.testing.assert_array_equal(got, want)
    sp.close()


def test_errors(gpu_context):
    b, m, _ = scenes.pile_1k()
    sp = GpuSpace(gpu_context, b, m)
    with pytest.raises(N.InvalidOperationException):  # no shapes uploaded
        sp.broad_phase(DT)
    sp.close()
    b, m, _, sh = scenes.make_pile(nx=3, ny=3, nz=3, narrow_phase=1, seed=2)
    sp = GpuSpace(gpu_context, b, m, shapes=sh)
    with pytest.raises(N.ArgumentException):
        sp.broad_phase(-1.0)
    sp.close()
