"""The device narrow phase against the oracle: box-box (face and edge cases,
axis-aligned and turned), box-sphere and sphere-sphere pairs whose contacts
are regenerated every step and matched by id, inside full steps, on every
path (graph, persistent, island groups), through record round trips, and the
errors the boundary reports."""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, default_settings

from parity import DT, STEP_TOL, Pair

pytestmark = pytest.mark.gpu


def _exact_contacts(p):
    gm, _ = p.gpu.download_constraints()
    om, _ = p.oracle.get_constraints()
    for f in ("contact_count", "contact_order", "sliding_axis", "sliding_impulse", "twist_impulse"):
        np.testing.assert_array_equal(gm[f], om[f], err_msg=f)
    for f in ("position", "normal", "penetration_depth", "id", "penetration_impulse"):
        np.testing.assert_array_equal(gm["contacts"][f], om["contacts"][f], err_msg=f)
    return gm


def _random_quats(n, rng, spread):
    axis = rng.normal(size=(n, 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    ang = rng.uniform(-spread, spread, n)
    q = np.concatenate([axis * np.sin(ang / 2)[:, None], np.cos(ang / 2)[:, None]], axis=1)
    return q.astype(np.float32)


def _all_pairs(bodies, shapes, margin=0.1):
    """Every pair whose bounding spheres come within `margin`, as empty
    GENERATED manifolds (the box first in box-sphere pairs)."""
    c = bodies["position"].astype(np.float64)
    r = np.where(shapes["type"] == N.SHAPE_BOX, np.linalg.norm(shapes["size"], axis=1), shapes["size"][:, 0])
    pairs = []
    n = len(bodies)
    for i in range(n):
        d = np.linalg.norm(c[i + 1:] - c[i], axis=1)
        for j in np.flatnonzero(d <= r[i] + r[i + 1:] + margin) + i + 1:
            if not (bodies["is_dynamic"][i] or bodies["is_dynamic"][j]):
                continue
            a, b = i, int(j)
            if shapes["type"][a] == N.SHAPE_SPHERE and shapes["type"][b] == N.SHAPE_BOX:
                a, b = b, a
            pairs.append((a, b))
    m = np.zeros(len(pairs), N.MANIFOLD_DTYPE)
    for k, (a, b) in enumerate(pairs):
        m[k]["body_a"], m[k]["body_b"] = a, b
    m["flags"] = N.MANIFOLD_ACTIVE | N.MANIFOLD_SOLVER_RULE | N.MANIFOLD_GENERATED
    m["kinetic_friction"] = m["static_friction"] = 0.5
    return m


def _jumble(seed=3, n=240, spread=np.pi, sphere_every=4):
    """Boxes and spheres at random orientations packed into overlapping
    neighbourhoods above a ground box: face, edge and corner contacts of every
    kind, deep and shallow."""
    rng = np.random.default_rng(seed)
    b, _, _, sh = scenes.make_pile(nx=8, ny=4, nz=8, spacing=0.9, size_min=0.5, size_max=1.1, jitter=0.15,
                                   narrow_phase=1, seed=seed)
    b = b[:n + 1].copy()
    sh = sh[:n + 1].copy()
    dyn = np.arange(1, len(b))
    b["orientation"][dyn] = _random_quats(len(dyn), rng, spread)
    b["position"][dyn] += rng.uniform(-0.08, 0.08, (len(dyn), 3)).astype(np.float32)
    spheres = dyn[::sphere_every]
    sh["type"][spheres] = N.SHAPE_SPHERE
    sh["size"][spheres, 0] = 0.45
    sh["size"][spheres, 1:] = 0
    return b, _all_pairs(b, sh), sh


def test_pile_narrow_phase_every_step(gpu_context):
    b, m, _, sh = scenes.make_pile(nx=6, ny=6, nz=6, narrow_phase=1, seed=21)
    p = Pair(gpu_context, b, m, settings=default_settings(), shapes=sh)
    for step in range(10):
        p.step()
        errs, exact = p.compare()
        assert exact, (step, errs)
        gm = _exact_contacts(p)
    assert gm["contact_count"].sum() > 0
    p.close()


def test_jumble_every_step(gpu_context):
    """Turned boxes and spheres: edge-edge, clipped faces, pruned manifolds."""
    b, m, sh = _jumble()
    p = Pair(gpu_context, b, m, settings=default_settings(), shapes=sh)
    for step in range(12):
        p.step()
        errs, exact = p.compare()
        assert exact, (step, errs)
        _exact_contacts(p)
    p.close()


def test_jumble_sixty_steps_groups_off_and_persistent(gpu_context):
    b, m, sh = _jumble(seed=5)
    runs = []
    for policy, mode in (((0, 1024, 4096, 64, 0), N.MODE_GRAPH), (None, N.MODE_PERSISTENT), (None, N.MODE_GRAPH)):
        p = Pair(gpu_context, b, m, settings=default_settings(), shapes=sh, group_policy=policy, mode=mode)
        p.step(steps=60)
        errs, exact = p.compare()
        assert exact, (policy, mode, errs)
        runs.append(_exact_contacts(p))
        p.close()
    for r in runs[1:]:
        np.testing.assert_array_equal(r["contacts"], runs[0]["contacts"])


def test_towers_with_spheres(gpu_context):
    b, m, _, sh = scenes.make_tower(300, seed=8, sphere_fraction=0.5, narrow_phase=1)
    assert (sh["type"] == N.SHAPE_SPHERE).any()
    p = Pair(gpu_context, b, m, settings=default_settings(), shapes=sh)
    for step in range(8):
        p.step()
        errs, exact = p.compare()
        assert exact, (step, errs)
        _exact_contacts(p)
    p.close()


def test_collide_stage_alone_and_mixed_with_frozen_manifolds(gpu_context):
    """STEP_COLLIDE alone, and GENERATED manifolds beside refreshed ones."""
    b, m, _, sh = scenes.make_pile(nx=4, ny=5, nz=4, narrow_phase=1, seed=22)
    fb, fm, _ = scenes.make_pile(nx=4, ny=5, nz=4, seed=22)
    assert len(fb) == len(b)
    mixed = np.concatenate([m[: len(m) // 2], fm[len(fm) // 2:]])
    for flags in (N.STEP_COLLIDE, N.STEP_ALL):
        p = Pair(gpu_context, b, mixed, settings=default_settings(), shapes=sh)
        p.step(flags=flags, steps=3)
        errs, exact = p.compare()
        assert exact, (flags, errs)
        _exact_contacts(p)
        p.close()


def test_records_round_trip_and_resume(gpu_context):
    """Downloading and re-uploading the records mid-run (contact_order
    included) continues bit for bit."""
    b, m, sh = _jumble(seed=9, n=120)
    st = default_settings()
    gpu_context.set_settings(st)
    ref = GpuSpace(gpu_context, b, m, shapes=sh)
    for _ in range(6):
        ref.step(DT)
    cut = GpuSpace(gpu_context, b, m, shapes=sh)
    for _ in range(3):
        cut.step(DT)
    mb = cut.download_bodies(b.copy())
    mm, _ = cut.download_constraints(m.copy())
    again = GpuSpace(gpu_context, mb, mm, shapes=sh)
    for _ in range(3):
        again.step(DT)
    rb, rm = ref.download_bodies(b.copy()), ref.download_constraints(m.copy())[0]
    ab, am = again.download_bodies(b.copy()), again.download_constraints(m.copy())[0]
    np.testing.assert_array_equal(rb["linear_velocity"], ab["linear_velocity"])
    np.testing.assert_array_equal(rm["contacts"], am["contacts"])
    np.testing.assert_array_equal(rm["contact_order"], am["contact_order"])
    for s in (ref, cut, again):
        s.close()


def test_boundary_errors(gpu_context):
    b, m, _, sh = scenes.make_pile(nx=3, ny=3, nz=3, narrow_phase=1, seed=23)
    gpu_context.set_settings(default_settings())
    with pytest.raises(N.BepuError):  # GENERATED manifolds need shapes first
        GpuSpace(gpu_context, b, m)
    sp = GpuSpace(gpu_context, b, m, shapes=sh)
    bad = sh.copy()
    bad["size"][1, 0] = -1
    with pytest.raises(N.BepuError):
        sp.upload_shapes(bad)
    bad = sh.copy()
    bad["type"][m["body_a"][0]] = N.SHAPE_NONE
    with pytest.raises(N.BepuError):  # breaks a GENERATED pair
        sp.upload_shapes(bad)
    sph = sh.copy()
    sph["type"][1:] = N.SHAPE_SPHERE
    sph["size"][1:, 0] = 0.5
    sp2 = GpuSpace(gpu_context, b, np.zeros(0, N.MANIFOLD_DTYPE), shapes=sph)
    swapped = m[m["body_a"] == 0].copy()
    swapped["body_a"], swapped["body_b"] = swapped["body_b"].copy(), swapped["body_a"].copy()
    with pytest.raises(N.BepuError):  # a sphere as body_a against a box
        sp2.upload_constraints(swapped)
    order = m.copy()
    order["contact_count"][0] = 2
    order["contact_order"][0] = 0xE4 ^ 0b0000  # entries 0, 0: not a permutation
    with pytest.raises(N.BepuError):
        sp.upload_constraints(order)
    toggled = m.copy()
    toggled["flags"][0] &= ~np.uint32(N.MANIFOLD_GENERATED)
    with pytest.raises(N.BepuError):  # update_manifolds keeps the GENERATED set
        sp.update_manifolds(toggled)
    sp.step(DT)
    sp.close()
    sp2.close()


def test_pile_64k_collide_full_size_two_steps(gpu_context):
    """The full narrow-phase workload (65,536 pairs of the 65,536-box pile)
    against the oracle for two steps."""
    b, m, _, sh = scenes.pile_64k_collide()
    p = Pair(gpu_context, b, m, settings=default_settings(), shapes=sh)
    p.step(steps=2)
    errs, exact = p.compare()
    assert exact, errs
    gm = _exact_contacts(p)
    assert gm["contact_count"].sum() > 250000
    p.close()
