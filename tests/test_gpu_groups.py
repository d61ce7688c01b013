"""Island groups (whole steps of small islands in one CTA) against the oracle,
alone and mixed with the colour-sweep path."""
import numpy as np
import pytest

from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, profile_step

from parity import DT, Pair

pytestmark = pytest.mark.gpu

POLICIES = {
    "sweep": (0, 1024, 4096, 256, 0),    # everything on the colour-sweep path
    "groups": (1, 1024, 4096, 256, 0),   # default: islands up to 1024 bodies in groups
    "mixed": (1, 24, 4096, 64, 0),       # small islands in groups, larger ones on the sweep path
    "narrow": (1, 1024, 4096, 256, 32),  # one warp per group: every colour loops
}


@pytest.mark.parametrize("policy", list(POLICIES))
def test_pile_1k_policies(gpu_context, policy):
    b, m, _ = scenes.pile_1k()
    p = Pair(gpu_context, b, m, group_policy=POLICIES[policy])
    p.step(steps=20)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


@pytest.mark.parametrize("policy", ["groups", "mixed"])
def test_towers_policies(gpu_context, policy):
    b, m, _ = scenes.make_tower(1200, seed=17)
    p = Pair(gpu_context, b, m, group_policy=POLICIES[policy])
    p.step(steps=20)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


def test_pile_64k_in_groups(gpu_context):
    b, m, _ = scenes.pile_64k()
    p = Pair(gpu_context, b, m, group_policy=POLICIES["groups"])
    prof = profile_step(p.gpu, DT, N.STEP_ALL)
    p.oracle.step(DT, N.STEP_ALL, 1)
    assert prof["groups"] > 0 and prof["solve_launches"] == 0  # every column is a small island
    p.step(steps=2)
    errs, exact = p.compare()
    assert exact, errs
    p.close()


def test_census_counts_the_same_work_on_both_paths(gpu_context):
    b, m, _ = scenes.pile_1k(seed=3)
    counts = {}
    for name in ("sweep", "groups"):
        sp = GpuSpace(gpu_context, b, m, group_policy=POLICIES[name])
        prof = profile_step(sp, DT, N.STEP_ALL)
        counts[name] = (prof["solve_manifold_visits"], prof["solve_algorithmic_bytes"])
        sp.close()
    assert counts["sweep"] == counts["groups"] and counts["sweep"][0] > 0


def test_group_policy_validation(gpu_context):
    b, m, _ = scenes.pile_1k()
    sp = GpuSpace(gpu_context, b, m)
    with pytest.raises(N.ArgumentException):
        sp.set_group_policy(1, 5000, 4096, 256, 0)
    with pytest.raises(N.ArgumentException):
        sp.set_group_policy(1, 1024, 4096, 256, 33)
    sp.close()
