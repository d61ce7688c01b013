"""The oracle's group continuation records: a group's motors and further
limits as extra children of its SolverGroup (SolverGroup.cs:88-165), after
the group's own children in the order its constructor Adds them.

SolverGroup.SolveIteration runs each active child's SolveUpdateable in order
and keeps the group active while any child is; Solver.UnsafeSolveIteration
applies the same iteration and zero-impulse rules to a joint of its own
(Solver.cs:285-314).  So, in list order, a group whose extra children are
continuation records performs exactly the operations of the same group
followed by those children as separate joints: the two runs agree bit for bit.
The children's own arithmetic is pinned by the closed forms in
test_oracle_joints.py.
"""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import default_settings

from joint_records import GROUP_CHILDREN, as_separate_children, with_group_children

DT = np.float32(1 / 60)


def _chains(seed, chains=10, links=10, loose=30):
    return scenes.make_chain(chains=chains, links=links, loose_bodies=loose, seed=seed,
                             region=np.array([24.0, 10.0, 24.0], np.float32))


def _settings(iterations=10):
    s = default_settings()
    s["iteration_limit"] = iterations
    return s


def _run(b, m, j, steps):
    o = oracle.OracleSpace(_settings(), b, m, j)
    o.step(DT, steps=steps)
    ob, (om, oj) = o.get_bodies(), o.get_constraints()
    o.close()
    return ob, om, oj


def _assert_same(x, y):
    xb, xm, xj = x
    yb, ym, yj = y
    for f in ("position", "orientation", "linear_velocity", "angular_velocity"):
        np.testing.assert_array_equal(xb[f], yb[f], err_msg=f)
    np.testing.assert_array_equal(xm["contacts"]["penetration_impulse"], ym["contacts"]["penetration_impulse"])
    np.testing.assert_array_equal(xj["impulse"], yj["impulse"])


@pytest.mark.parametrize("head", list(GROUP_CHILDREN))
def test_continuations_solve_as_children_after_their_group(head):
    b, m, j = _chains(seed=7 + head)
    jc = with_group_children(b, j, 7 + head, heads=(head,), keep=1.0)
    cont = (jc["flags"] & N.JOINT_GROUP_CONTINUATION) != 0
    assert cont.sum() >= 4 * len(GROUP_CHILDREN[head])
    got = _run(b, m, jc, 12)
    _assert_same(got, _run(b, m, as_separate_children(jc), 12))
    # the children did work: their impulses moved off zero
    assert np.count_nonzero(got[2]["impulse"][cont][:, :3]) > 0


def test_inactive_children_and_groups():
    """An inactive child takes no part; an inactive group takes its children
    out with it (SolverGroup.UpdateSolverActivity, SolverGroup.cs:52-68)."""
    b, m, j = _chains(seed=11)
    jc = with_group_children(b, j, 11, keep=0.8, inactive_children=0.3, inactive_groups=0.25)
    cont = (jc["flags"] & N.JOINT_GROUP_CONTINUATION) != 0
    got = _run(b, m, jc, 8)
    _assert_same(got, _run(b, m, as_separate_children(jc), 8))
    # children that are off (or whose group is off) keep their impulses
    sep = as_separate_children(jc)
    off = cont & ((sep["flags"] & N.JOINT_ACTIVE) == 0)
    assert off.any()
    np.testing.assert_array_equal(got[2]["impulse"][off], jc["impulse"][off])


def test_colouring_gives_continuations_their_group_colour():
    """A continuation takes its group record's colour and claims nothing: the
    other entries' colours are those of the list without it."""
    b, m, j = _chains(seed=13)
    jc = with_group_children(b, j, 13, keep=1.0)
    cont = (jc["flags"] & N.JOINT_GROUP_CONTINUATION) != 0
    col, order, k = oracle.colour(b, m, jc)
    idx = np.flatnonzero(cont)
    assert len(idx)
    np.testing.assert_array_equal(col[idx], col[idx - 1])
    keep = np.concatenate([~cont, np.ones(len(m), bool)])
    col2, _, _ = oracle.colour(b, m, jc[~cont])
    np.testing.assert_array_equal(col[keep], col2)
    # colour-major order with list order inside a colour: a group's
    # continuations directly follow it
    pos = np.empty_like(order)
    pos[order] = np.arange(len(order))
    np.testing.assert_array_equal(pos[idx], pos[idx - 1] + 1)


def test_oracle_rejects_a_continuation_without_a_group():
    b, m, j = _chains(seed=17)
    jc = with_group_children(b, j, 17, keep=1.0)
    bad = jc.copy()
    bad["flags"][0] |= N.JOINT_GROUP_CONTINUATION
    with pytest.raises(ValueError):
        oracle.OracleSpace(_settings(), b, m, bad)
