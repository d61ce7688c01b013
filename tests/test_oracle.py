"""CPU tests of the oracle: the reference's known-answer property for
PermutationMapper, hand-derived single-contact answers, and the invariants of
the restated solver (Solver.cs:239-314)."""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import colour_list, default_settings

DT = np.float32(1 / 60)


def test_prime_table_pinned():
    # BEPUutilities/PermutationMapper.cs:49-104 holds 503 primes; first and last pinned.
    assert oracle.prime_count() == 503
    assert oracle.permutation_map(0, 1, 1_000_000_007) == 818660357
    assert oracle.permutation_map(502, 1, 2_000_000_000) == (475092199 + 475092199 * 502) % 2_000_000_000


def test_permutation_mapper_bijection():
    # PermutationTestDemo.cs:82-127: for set size 250, every block of 250
    # consecutive indices maps onto [0, 250) without repeats, for every index.
    set_size = 250
    for perm in list(range(0, 1200, 7)) + [149_999]:
        mapped = {oracle.permutation_map(perm, i, set_size) for i in range(set_size)}
        assert mapped == set(range(set_size))
        block2 = {oracle.permutation_map(perm, i, set_size) for i in range(set_size, 2 * set_size)}
        assert block2 == set(range(set_size))


def test_permutation_demo_full_run():
    # PermutationTestDemo.cs:88-115 as the reference runs it: 150,000 permutation
    # indices, set size 250, each mapping a permutation (the demo throws otherwise).
    first_bad, distinct = oracle.permutation_check(150_000, 250)
    assert first_bad == -1
    # The mapping is p * (i + k) mod 250 with p one of the 503 primes (all odd and
    # none a multiple of 5, so units mod 250): at most 100 multipliers x 250 shifts.
    assert 0 < distinct <= 100 * 250


def test_permutation_mapper_formula():
    # GetMappedIndex = (index * prime + prime * permutationIndex) mod setSize
    primes0 = 818660357
    for i in range(20):
        assert oracle.permutation_map(0, i, 97) == (i * primes0) % 97


def _one_contact_scene(depth=0.0, mass=1.0, vy=0.0):
    bodies = np.zeros(2, N.BODY_DTYPE)
    bodies["orientation"][:, 3] = 1
    bodies["linear_damping"] = 0.03
    bodies["angular_damping"] = 0.15
    bodies[1]["position"] = (0, 0.5, 0)
    bodies[1]["is_dynamic"] = 1
    bodies[1]["inverse_mass"] = np.float32(1) / np.float32(mass)
    bodies[1]["local_inverse_inertia"] = np.diag([6.0, 6.0, 6.0]).astype(np.float32).ravel() / mass
    bodies[1]["linear_velocity"] = (0, vy, 0)
    m = np.zeros(1, N.MANIFOLD_DTYPE)
    m["body_a"], m["body_b"], m["contact_count"] = 0, 1, 1
    m["flags"] = N.MANIFOLD_ACTIVE | N.MANIFOLD_SOLVER_RULE
    m["kinetic_friction"] = m["static_friction"] = 0.36
    c = m[0]["contacts"][0]
    c["position"] = (0, 0, 0)
    c["normal"] = (0, 1, 0)
    c["penetration_depth"] = depth
    c["base_penetration_depth"] = depth
    c["local_offset_b"] = (0, -0.5, 0)
    m[0]["contacts"][0] = c
    return bodies, m


def test_single_contact_known_answer():
    """A resting unit box with one centred contact: after the force update
    v = (g dt) * 0.97^dt; one penetration solve gives
    lambda = -v / (1 + softness), softness = 0.001 * 1 * 60 (ContactPenetrationConstraint.cs:184-187)."""
    s = default_settings()
    s["iteration_limit"] = 1
    bodies, m = _one_contact_scene()
    o = oracle.OracleSpace(s, bodies, m)
    o.step(DT, N.STEP_FORCES | N.STEP_SOLVE, 1)
    b = o.get_bodies()
    mo, _ = o.get_constraints()
    f32 = np.float32
    v = f32(f32(-9.81) * DT) + f32(0)
    v = f32(v * f32(np.float64(f32(1) - f32(0.03)) ** np.float64(DT)))
    softness = f32(f32(f32(0.001) * f32(1)) * f32(f32(1) / DT))
    v2i = f32(f32(-1) / f32(softness + f32(1)))
    rv = v  # relative velocity -vB . linearA with linearA = -n = (0, -1, 0); ground at rest
    lam = f32(f32(rv - f32(0) + f32(softness * f32(0))) * v2i)
    acc = max(f32(0), lam)
    assert mo[0]["contacts"][0]["penetration_impulse"] == pytest.approx(float(acc), rel=1e-6)
    assert b[1]["linear_velocity"][1] == pytest.approx(float(v + acc), rel=1e-5)
    # no tangential motion, no friction impulse, no spin
    assert np.all(b[1]["angular_velocity"] == 0)
    assert mo[0]["sliding_impulse"][0] == 0 and mo[0]["sliding_impulse"][1] == 0


def test_separated_contact_applies_nothing():
    # Negative depth and a slow approach: bias = depth / dt keeps lambda clamped at 0.
    s = default_settings()
    bodies, m = _one_contact_scene(depth=-0.05, vy=0.0)
    o = oracle.OracleSpace(s, bodies, m)
    o.step(DT, N.STEP_SOLVE, 1)
    mo, _ = o.get_constraints()
    assert mo[0]["contacts"][0]["penetration_impulse"] == 0.0


def test_kinematic_only_manifold_is_inactive():
    s = default_settings()
    bodies, m = _one_contact_scene(vy=-1.0)
    bodies[1]["is_dynamic"] = 0
    o = oracle.OracleSpace(s, bodies, m)
    o.step(DT, N.STEP_SOLVE, 1)
    assert o.last_child_solves() == 0


def test_early_out_counts():
    """A constraint whose impulse stays below minimumImpulse deactivates after
    minimumIterationCount + 1 zero iterations (SolverGroup.cs:127-136)."""
    s = default_settings()
    s["iteration_limit"] = 10
    bodies, m = _one_contact_scene(depth=-0.05)
    o = oracle.OracleSpace(s, bodies, m)
    o.step(DT, N.STEP_SOLVE, 1)
    # 3 children (1 penetration, sliding, twist), each solved twice before it
    # deactivates; the group then has no active child.
    assert o.last_child_solves() == 6


def test_colouring_matches_restatement_and_is_conflict_free():
    b, m, _ = scenes.pile_1k()
    col, order, k = colour_list(b, m)
    col2, order2, k2 = oracle.colour(b, m)
    assert k == k2
    np.testing.assert_array_equal(col, col2)
    np.testing.assert_array_equal(order, order2)
    dyn = b["is_dynamic"] != 0
    for c in range(k):
        members = np.nonzero(col == c)[0]
        seen = set()
        for u in members:
            for body in (m[u]["body_a"], m[u]["body_b"]):
                if body >= 0 and dyn[body]:
                    assert body not in seen
                    seen.add(body)
    # order is a stable colour sort
    assert np.all(np.diff(col[order]) >= 0)
    for c in range(k):
        idx = order[col[order] == c]
        assert np.all(np.diff(idx) > 0)


def test_colouring_edge_cases():
    b, m, _ = scenes.pile_1k()
    col, order, k = colour_list(b, m[:0])
    assert k == 0 and len(col) == 0
    bad = m[:3].copy()
    bad["body_b"][1] = len(b) + 5
    with pytest.raises(ValueError):
        colour_list(b, bad)


def _approach_residual(bodies, manifolds):
    """RMS over contacts of the approach speed along the normal left after a
    step (the velocity residual of the penetration constraints: relative
    velocity of B against A at the contact, negative when approaching)."""
    v = bodies["linear_velocity"].astype(np.float64)
    w = bodies["angular_velocity"].astype(np.float64)
    p = bodies["position"].astype(np.float64)
    out = []
    for mi in manifolds:
        a, bb = mi["body_a"], mi["body_b"]
        for k in range(mi["contact_count"]):
            c = mi["contacts"][k]
            x, n = c["position"].astype(np.float64), c["normal"].astype(np.float64)
            va = v[a] + np.cross(w[a], x - p[a]) if a >= 0 else np.zeros(3)
            vb = v[bb] + np.cross(w[bb], x - p[bb]) if bb >= 0 else np.zeros(3)
            out.append(min(float(np.dot(vb - va, n)), 0.0))
    return float(np.sqrt(np.mean(np.square(out))))


def test_reference_order_and_colour_order_reach_equal_residual():
    """Reference order (PermutationMapper) and colour order are both
    Gauss-Seidel sweeps over the same constraints but in different orders, so
    their states differ; after 60 steps both leave the pile with the same
    small velocity residual (approach speed at the contacts within 25 % of
    each other and below 1 cm/s) and poses within 2 cm."""
    s = default_settings()
    b, m, _ = scenes.pile_1k()
    col, order, _ = colour_list(b, m)
    ref = oracle.OracleSpace(s, b, m)
    ref.set_order_mode(oracle.ORDER_PERMUTED, 0)
    colr = oracle.OracleSpace(s, b, m)
    colr.set_list_order(order)
    ref.step(DT, N.STEP_ALL, 60)
    colr.step(DT, N.STEP_ALL, 60)
    b1, b2 = ref.get_bodies(), colr.get_bodies()
    r1 = _approach_residual(b1, ref.get_constraints()[0])
    r2 = _approach_residual(b2, colr.get_constraints()[0])
    assert r1 < 0.01 and r2 < 0.01, (r1, r2)
    assert abs(r1 - r2) <= 0.25 * max(r1, r2), (r1, r2)
    assert np.abs(b1["position"] - b2["position"]).max() < 0.02
    assert np.abs(b1["linear_velocity"]).max() < 1.0 and np.abs(b2["linear_velocity"]).max() < 1.0


def test_multithreaded_baseline_runs():
    s = default_settings()
    b, m, _ = scenes.pile_1k()
    o = oracle.OracleSpace(s, b, m)
    o.set_order_mode(oracle.ORDER_PERMUTED, 0)
    o.step_multithreaded(DT, N.STEP_ALL, 3, 4)
    v = o.get_bodies()["linear_velocity"]
    assert np.isfinite(v).all() and np.abs(v).max() < 1.0


def test_float_sqrt_through_double_is_float_sqrt():
    """(float)Math.Sqrt((double)x) == IEEE sqrtf(x) for every float x: double
    has at least 2*24+2 significant bits, so the double rounding is innocuous
    (Figueroa 1995).  The device solver relies on this identity."""
    rng = np.random.default_rng(7)
    bits = rng.integers(0, 0x7f800000, size=2_000_000, dtype=np.uint32)  # every finite non-negative float
    x = bits.view(np.float32)
    edge = np.array([0.0, -0.0, 1e-45, 1.17549435e-38, 3.4028235e38, 1.0, 2.0, 0.25, np.inf], np.float32)
    x = np.concatenate([x, edge])
    via_double = np.sqrt(x.astype(np.float64)).astype(np.float32)
    direct = np.sqrt(x)
    np.testing.assert_array_equal(via_double.view(np.uint32), direct.view(np.uint32))
