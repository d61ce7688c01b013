"""The allocation-free step, bepugpu_step_noalloc, against the regular entry
points.

Some callers cannot allocate device memory themselves -- an engine plugin
whose host owns the device heap, or a process held to a memory budget fixed
in advance.  They hand the library records that already sit in device memory
and the library works in one fixed scratch array.  This test places the
records in device memory the way such a caller would (here through torch),
steps twice through the C ABI and checks each result against the regular
upload / step / download path on the same scene.  The file is named to be
collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, default_settings

from parity import DT, STEP_TOL, rel_err

pytestmark = pytest.mark.gpu


def _records_on_device(records: np.ndarray):
    import torch
    return torch.from_numpy(records.copy().view(np.uint8)).cuda()


def _step_noalloc(lib, settings, dev_bodies, nb, dev_manifolds, nm, flags=N.STEP_ALL):
    return lib.bepugpu_step_noalloc(N.ptr(settings), ctypes.c_void_p(dev_bodies.data_ptr()), nb,
                                    ctypes.c_void_p(dev_manifolds.data_ptr()), nm, float(DT), flags, None)


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
        gb = dev_b.cpu().numpy().view(N.BODY_DTYPE)
        gm = dev_m.cpu().numpy().view(N.MANIFOLD_DTYPE)
        eb, em = expected[call]
        np.testing.assert_array_equal(gm["contact_count"], em["contact_count"])
        np.testing.assert_array_equal(gm["contacts"]["id"], em["contacts"]["id"])
        for field in ("linear_velocity", "angular_velocity", "position", "orientation"):
            assert rel_err(gb[field], eb[field]) <= STEP_TOL, (call, field)
        assert rel_err(gm["contacts"]["penetration_impulse"], em["contacts"]["penetration_impulse"]) <= STEP_TOL
        assert rel_err(gm["sliding_impulse"], em["sliding_impulse"]) <= STEP_TOL
        assert rel_err(gm["twist_impulse"], em["twist_impulse"]) <= STEP_TOL


def test_noalloc_rejects_scenes_beyond_its_scratch():
    import torch
    settings = np.array(default_settings()).reshape(1)
    lib = N.load_gpu_library()
    tiny = torch.zeros(64, dtype=torch.uint8, device="cuda")
    st = _step_noalloc(lib, settings, tiny, N.NOALLOC_MAX_BODIES + 1, tiny, 0)
    assert st == N.INVALID_ARGUMENT
    st = _step_noalloc(lib, settings, tiny, 0, tiny, N.NOALLOC_MAX_MANIFOLDS + 1)
    assert st == N.INVALID_ARGUMENT
