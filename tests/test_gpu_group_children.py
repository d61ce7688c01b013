"""Group continuation records on the device against the oracle: a group's
motors and further limits solved inside the group's visit, after its own
children, on the colour-sweep path, in island groups and in the persistent
kernel; their colouring, record checks and resumption from records."""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, default_settings

from joint_records import GROUP_CHILDREN, with_group_children
from parity import DT, Pair

pytestmark = pytest.mark.gpu

GROUPS_ON = (1, 1024, 4096, 64, 0)
GROUPS_OFF = (0, 1024, 4096, 64, 0)


def _settings(iterations=15):
    s = default_settings()
    s["iteration_limit"] = iterations
    return s


def _chains(seed, chains=24, links=12, loose=120):
    return scenes.make_chain(chains=chains, links=links, loose_bodies=loose, seed=seed,
                             region=np.array([30.0, 12.0, 30.0], np.float32))


@pytest.mark.parametrize("head", list(GROUP_CHILDREN))
def test_each_group_with_its_children_every_step(gpu_context, head):
    b, m, j = _chains(seed=50 + head)
    j = with_group_children(b, j, 50 + head, heads=(head,), keep=1.0)
    assert (j["flags"] & N.JOINT_GROUP_CONTINUATION).any()
    p = Pair(gpu_context, b, m, j, settings=_settings(), group_policy=GROUPS_OFF)
    for step in range(5):
        p.step()
        errs, exact = p.compare()
        assert exact, (head, step, errs)
    p.close()


@pytest.mark.parametrize("policy,mode", [(GROUPS_OFF, N.MODE_GRAPH), (GROUPS_ON, N.MODE_GRAPH),
                                         (None, N.MODE_PERSISTENT)])
def test_group_children_sixty_steps_every_path(gpu_context, policy, mode):
    b, m, j = _chains(seed=61)
    j = with_group_children(b, j, 61, keep=0.7, inactive_children=0.15, inactive_groups=0.1)
    p = Pair(gpu_context, b, m, j, settings=_settings(), group_policy=policy, mode=mode)
    p.step(steps=60)
    errs, exact = p.compare()
    assert exact, (policy, mode, errs)
    p.close()


def test_colouring_matches_the_oracle(gpu_context):
    b, m, j = _chains(seed=62)
    j = with_group_children(b, j, 62, keep=1.0)
    sp = GpuSpace(gpu_context, b, m, j)
    col, order, k = sp.colouring()
    col2, order2, k2 = oracle.colour(b, m, j)
    np.testing.assert_array_equal(col, col2)
    np.testing.assert_array_equal(order, order2)
    assert k == k2
    idx = np.flatnonzero(j["flags"] & N.JOINT_GROUP_CONTINUATION)
    np.testing.assert_array_equal(col[idx], col[idx - 1])
    sp.close()


def test_continuation_records_checked(gpu_context):
    b, m, j = _chains(seed=63, chains=4, loose=0)
    j = with_group_children(b, j, 63, keep=1.0)
    idx = np.flatnonzero(j["flags"] & N.JOINT_GROUP_CONTINUATION)
    assert len(idx)
    cases = []
    bad = j.copy()  # the first record cannot continue anything
    bad["flags"][0] |= N.JOINT_GROUP_CONTINUATION
    cases.append(bad)
    bad = j.copy()  # a child the group does not take
    bad["type"][idx[0]] = N.JOINT_BALL_SOCKET
    cases.append(bad)
    bad = j.copy()  # other bodies than the group's
    bad["body_b"][idx[0]] = -1 if bad["body_b"][idx[0]] != -1 else 0
    cases.append(bad)
    # a fifth child: the first continuation repeated five times
    extra = np.repeat(j[idx[0]:idx[0] + 1], 5)
    cases.append(np.concatenate([j[:idx[0]], extra, j[idx[0] + 1:]]))
    for bad in cases:
        with pytest.raises(N.BepuError):
            GpuSpace(gpu_context, b, m, bad)


def test_group_children_resume_from_records(gpu_context):
    """Stepping, downloading the records, uploading them into a new scene and
    stepping on continues bit for bit like the uninterrupted run."""
    b, m, j = _chains(seed=64)
    j = with_group_children(b, j, 64, keep=1.0)
    gpu_context.set_settings(_settings())
    ref = GpuSpace(gpu_context, b, m, j)
    for _ in range(6):
        ref.step(float(DT))
    cut = GpuSpace(gpu_context, b, m, j)
    for _ in range(3):
        cut.step(float(DT))
    mb = cut.download_bodies(b.copy())
    mm, mj = cut.download_constraints(m.copy(), j.copy())
    again = GpuSpace(gpu_context, mb, mm, mj)
    for _ in range(3):
        again.step(float(DT))
    rb, ab = ref.download_bodies(b.copy()), again.download_bodies(b.copy())
    for f in ("position", "orientation", "linear_velocity", "angular_velocity"):
        np.testing.assert_array_equal(rb[f], ab[f], err_msg=f)
    np.testing.assert_array_equal(ref.download_constraints(m.copy(), j.copy())[1]["impulse"],
                                  again.download_constraints(m.copy(), j.copy())[1]["impulse"])
    for s in (ref, cut, again):
        s.close()
