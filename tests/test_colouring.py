"""Race freedom of the colour sweeps, checked on the host: inside one colour
no two constraints share a dynamic body (the bodies the reference locks,
SolverUpdateable.cs:151-160), so a colour's data-parallel sweep equals the
sequential Gauss-Seidel sweep over it; and the colour-sorted order keeps list
order inside a colour."""
import numpy as np
import pytest

from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import colour_list


def _check(bodies, manifolds, joints=None):
    colour, order, k = colour_list(bodies, manifolds, joints)
    nj = 0 if joints is None else len(joints)
    a = np.concatenate([joints["body_a"] if nj else np.zeros(0, np.int32), manifolds["body_a"]])
    b = np.concatenate([joints["body_b"] if nj else np.zeros(0, np.int32), manifolds["body_b"]])
    dyn = bodies["is_dynamic"] != 0
    for c in range(k):
        members = np.flatnonzero(colour == c)
        touched = []
        for u in members:
            for e in (a[u], b[u]):
                if e >= 0 and dyn[e]:
                    touched.append(e)
        assert len(touched) == len(set(touched)), f"colour {c} shares a dynamic body"
    # order: colour-major, list order inside a colour
    assert np.all(np.diff(colour[order]) >= 0)
    for c in range(k):
        inside = order[colour[order] == c]
        assert np.all(np.diff(inside) > 0)
    return k


@pytest.mark.parametrize("name", ["pile_1k", "towers", "chains"])
def test_colours_are_race_free(name):
    if name == "pile_1k":
        b, m, j = scenes.pile_1k()
    elif name == "towers":
        b, m, j = scenes.make_tower(600, seed=5)
    else:
        b, m, j = scenes.make_chain(chains=40, loose_bodies=200, seed=4,
                                    region=np.array([20.0, 10.0, 20.0], np.float32))
    k = _check(b, m, j if len(j) else None)
    assert k >= 2
