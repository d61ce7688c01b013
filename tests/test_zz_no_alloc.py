"""The allocation-free step, bepugpu_step_noalloc, against the regular entry
points and the oracle.

Some callers cannot allocate device memory themselves -- an engine plugin
whose host owns the device heap, or a process held to a memory budget fixed
in advance.  They hand the library records that already sit in device memory
and the library works in one fixed scratch array.  These tests place the
records in device memory the way such a caller would (here through torch),
step through the C ABI and check the results against the regular upload /
step / download path and against the oracle's colour-order run (the same
colouring: greedy in list order), on two calls in a row.  They also check
the refusals: sizes beyond the scratch, more than 128 colours, and records
the device rejects, which leave the caller's records unchanged.  The file is
named to be collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, colour_list, default_settings

from parity import DT, STEP_TOL, compare, rel_err

pytestmark = pytest.mark.gpu


def _records_on_device(records: np.ndarray):
    import torch
    return torch.from_numpy(records.copy().view(np.uint8)).cuda()


def _step_noalloc(lib, settings, dev_bodies, nb, dev_manifolds, nm, flags=N.STEP_ALL):
    return lib.bepugpu_step_noalloc(N.ptr(settings), ctypes.c_void_p(dev_bodies.data_ptr()), nb,
                                    ctypes.c_void_p(dev_manifolds.data_ptr()), nm, float(DT), flags, None)


def _host(dev, dtype):
    return dev.cpu().numpy().view(dtype)


def test_noalloc_matches_regular_step_on_two_calls(gpu_context):
    import torch
    settings = np.array(default_settings()).reshape(1)
    gpu_context.set_settings(settings[0])
    bodies, manifolds, _ = scenes.make_pile(nx=4, ny=4, nz=4, seed=21)
    assert len(bodies) <= N.NOALLOC_MAX_BODIES and len(manifolds) <= N.NOALLOC_MAX_MANIFOLDS

    regular = GpuSpace(gpu_context, bodies, manifolds)
    expected = []
    for _ in range(2):
        regular.step(DT, N.STEP_ALL)
        eb = regular.download_bodies(bodies.copy())
        em, _ = regular.download_constraints(manifolds.copy())
        expected.append((eb, em))
    regular.close()

    lib = N.load_gpu_library()
    dev_b = _records_on_device(bodies)
    dev_m = _records_on_device(manifolds)
    torch.cuda.synchronize()
    for call in range(2):
        st = _step_noalloc(lib, settings, dev_b, len(bodies), dev_m, len(manifolds))
        assert st == N.OK, N.STATUS_NAMES[st]
        gb = _host(dev_b, N.BODY_DTYPE)
        gm = _host(dev_m, N.MANIFOLD_DTYPE)
        eb, em = expected[call]
        np.testing.assert_array_equal(gm["contact_count"], em["contact_count"])
        np.testing.assert_array_equal(gm["contacts"]["id"], em["contacts"]["id"])
        for field in ("linear_velocity", "angular_velocity", "position", "orientation"):
            assert rel_err(gb[field], eb[field]) <= STEP_TOL, (call, field)
        assert rel_err(gm["contacts"]["penetration_impulse"], em["contacts"]["penetration_impulse"]) <= STEP_TOL
        assert rel_err(gm["sliding_impulse"], em["sliding_impulse"]) <= STEP_TOL
        assert rel_err(gm["twist_impulse"], em["twist_impulse"]) <= STEP_TOL


def _oracle_colour_order(settings, bodies, manifolds):
    _, order, _ = colour_list(bodies, manifolds)
    o = oracle.OracleSpace(settings[0], bodies, manifolds)
    o.set_list_order(order)
    o.set_order_mode(oracle.ORDER_IDENTITY)
    return o


@pytest.mark.parametrize("flags", [N.STEP_ALL, N.STEP_FORCES | N.STEP_SOLVE, N.STEP_SOLVE,
                                   N.STEP_REFRESH_CONTACTS | N.STEP_POSITIONS, N.STEP_DEACTIVATION])
@pytest.mark.parametrize("mover", [False, True])
def test_noalloc_bit_exact_against_oracle(flags, mover):
    """Two calls in a row give the oracle's colour-order bits, for subsets of
    the stages and with a moving kinematic ground."""
    import torch
    settings = np.array(default_settings()).reshape(1)
    bodies, manifolds, _ = scenes.make_pile(nx=5, ny=6, nz=5, seed=33)
    assert len(bodies) <= N.NOALLOC_MAX_BODIES and len(manifolds) <= N.NOALLOC_MAX_MANIFOLDS
    if mover:
        ground = int(np.flatnonzero(bodies["is_dynamic"] == 0)[0])
        bodies[ground]["linear_velocity"] = (0.2, 0.0, -0.1)
        bodies[ground]["angular_velocity"] = (0.0, 0.03, 0.0)
    o = _oracle_colour_order(settings, bodies, manifolds)
    lib = N.load_gpu_library()
    dev_b = _records_on_device(bodies)
    dev_m = _records_on_device(manifolds)
    torch.cuda.synchronize()
    for call in range(2):
        st = _step_noalloc(lib, settings, dev_b, len(bodies), dev_m, len(manifolds), flags)
        assert st == N.OK, N.STATUS_NAMES[st]
        o.step(DT, flags)
        gb, gm = _host(dev_b, N.BODY_DTYPE), _host(dev_m, N.MANIFOLD_DTYPE)
        ob = o.get_bodies()
        om, _ = o.get_constraints()
        errs, exact = compare(gb, gm, ob, om)
        assert exact, (call, errs)
        for f in ("position", "orientation", "activity", "velocity_time_below_limit", "previous_velocity"):
            assert gb[f].tobytes() == ob[f].tobytes(), (call, f)
        assert gm["sliding_impulse"].tobytes() == om["sliding_impulse"].tobytes()
        assert gm["twist_impulse"].tobytes() == om["twist_impulse"].tobytes()
    o.close()


def test_noalloc_rejects_scenes_beyond_its_scratch():
    import torch
    settings = np.array(default_settings()).reshape(1)
    lib = N.load_gpu_library()
    tiny = torch.zeros(64, dtype=torch.uint8, device="cuda")
    st = _step_noalloc(lib, settings, tiny, N.NOALLOC_MAX_BODIES + 1, tiny, 0)
    assert st == N.INVALID_ARGUMENT
    st = _step_noalloc(lib, settings, tiny, 0, tiny, N.NOALLOC_MAX_MANIFOLDS + 1)
    assert st == N.INVALID_ARGUMENT
    bad = settings.copy()
    bad["iteration_limit"] = 65536  # the bound bepugpu_set_settings applies
    st = _step_noalloc(lib, bad, tiny, 0, tiny, 0)
    assert st == N.INVALID_ARGUMENT


def _star(n_manifolds):
    """One dynamic body touching `n_manifolds` kinematic bodies: every manifold
    shares the dynamic body, so the list needs one colour per manifold."""
    bodies, manifolds, _ = scenes.make_pile(nx=1, ny=1, nz=1, seed=2)
    dyn = int(np.flatnonzero(bodies["is_dynamic"] != 0)[0])
    wall = bodies[np.flatnonzero(bodies["is_dynamic"] == 0)[0]]
    b = np.concatenate([bodies[dyn:dyn + 1], np.repeat(wall[None], n_manifolds)])
    m = np.repeat(manifolds[:1], n_manifolds)
    m["body_a"] = 0
    m["body_b"] = np.arange(1, n_manifolds + 1)
    return b, m


def test_noalloc_colour_limit():
    import torch
    settings = np.array(default_settings()).reshape(1)
    lib = N.load_gpu_library()
    for n, want in ((128, N.OK), (129, N.INVALID_OPERATION)):
        b, m = _star(n)
        assert colour_list(b, m)[2] == n
        dev_b, dev_m = _records_on_device(b), _records_on_device(m)
        torch.cuda.synchronize()
        st = _step_noalloc(lib, settings, dev_b, len(b), dev_m, len(m))
        assert st == want, (n, N.STATUS_NAMES[st])
        if want != N.OK:  # refused before any record was written
            assert _host(dev_b, N.BODY_DTYPE).tobytes() == b.tobytes()
            assert _host(dev_m, N.MANIFOLD_DTYPE).tobytes() == m.tobytes()


@pytest.mark.parametrize("field,value", [("body_b", 10 ** 6), ("contact_count", 5), ("body_a", -2), ("same", 0),
                                         ("flags", N.MANIFOLD_ACTIVE | N.MANIFOLD_SOLVER_RULE | N.MANIFOLD_NONCONVEX)])
def test_noalloc_device_side_validation(field, value):
    """A bad manifold record is caught on the device (the host only checks
    sizes): INVALID_ARGUMENT, the caller's records untouched, and the next
    valid call succeeds (the error word does not stick)."""
    import torch
    settings = np.array(default_settings()).reshape(1)
    bodies, manifolds, _ = scenes.make_pile(nx=3, ny=3, nz=3, seed=7)
    bad = manifolds.copy()
    if field == "same":
        bad["body_b"][4] = bad["body_a"][4]
    else:
        bad[field][4] = value
    lib = N.load_gpu_library()
    dev_b, dev_m = _records_on_device(bodies), _records_on_device(bad)
    torch.cuda.synchronize()
    st = _step_noalloc(lib, settings, dev_b, len(bodies), dev_m, len(bad))
    assert st == N.INVALID_ARGUMENT, N.STATUS_NAMES[st]
    assert _host(dev_b, N.BODY_DTYPE).tobytes() == bodies.tobytes()
    assert _host(dev_m, N.MANIFOLD_DTYPE).tobytes() == bad.tobytes()
    good = _records_on_device(manifolds)
    torch.cuda.synchronize()
    st = _step_noalloc(lib, settings, dev_b, len(bodies), good, len(manifolds))
    assert st == N.OK, N.STATUS_NAMES[st]
