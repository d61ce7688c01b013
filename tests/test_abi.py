"""The C-ABI library loads on a machine without a GPU and exports every symbol
the headers declare; record layouts match the binding."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from bepuphysics1_gb300 import native as N

ROOT = Path(__file__).resolve().parents[1]


def _declared(header: str, prefix: str):
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(" + prefix + r"_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(str(N.LIB_DIR / "libbepugpu.so"))
    names = _declared("bepugpu.h", "bepugpu")
    assert "bepugpu_step" in names and "bepugpu_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    scene = ctypes.CDLL(str(N.LIB_DIR / "libbepuscenes.so"))
    names = _declared("bepuscenes.h", "bepuscene")
    missing = [n for n in names if not hasattr(scene, n)]
    assert not missing, missing


def test_binding_covers_header():
    names = set(_declared("bepugpu.h", "bepugpu"))
    assert names <= set(N.GPU_EXPORTS), names - set(N.GPU_EXPORTS)


def test_record_sizes():
    lib = N.load_gpu_library()
    assert lib.bepugpu_abi_version() == 12
    assert lib.bepugpu_record_size(0) == N.SETTINGS_DTYPE.itemsize
    assert lib.bepugpu_record_size(1) == N.BODY_DTYPE.itemsize == 116
    assert lib.bepugpu_record_size(2) == N.CONTACT_DTYPE.itemsize == 80
    assert lib.bepugpu_record_size(3) == N.MANIFOLD_DTYPE.itemsize
    assert lib.bepugpu_record_size(4) == N.JOINT_DTYPE.itemsize
    assert lib.bepugpu_record_size(5) == N.BODY_STATE_DTYPE.itemsize == 64
    assert lib.bepugpu_record_size(6) == N.MANIFOLD_STATE_DTYPE.itemsize == 80
    assert lib.bepugpu_record_size(99) == 0


def test_default_settings_are_the_reference_defaults():
    from bepuphysics1_gb300.solver import default_settings
    s = default_settings()
    assert s["iteration_limit"] == 10                       # Solver.cs:15
    assert s["minimum_impulse"] == np.float32(0.001)        # SolverSettings.cs:62
    assert s["minimum_iteration_count"] == 1                # SolverSettings.cs:70
    assert s["softness"] == np.float32(0.001)               # CollisionResponseSettings.cs:43
    assert s["penetration_recovery_stiffness"] == np.float32(0.2)
    assert s["maximum_penetration_recovery_speed"] == 2
    assert s["static_friction_velocity_threshold"] == np.float32(0.2)
    assert s["allowed_penetration"] == np.float32(0.01)     # CollisionDetectionSettings.cs:74
    assert tuple(s["gravity"]) == (0, np.float32(-9.81), 0)
    assert s["use_stabilization"] == 1                      # DeactivationManager.cs:60
    assert s["velocity_lower_limit"] == np.float32(0.26)    # DeactivationManager.cs:18
    assert s["low_velocity_time_minimum"] == 1              # DeactivationManager.cs:20


def test_create_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    lib = N.load_gpu_library()
    h = ctypes.c_void_p()
    st = lib.bepugpu_create(0, None, ctypes.byref(h))
    assert st == N.CUDA_ERROR and not h.value


def test_scene_source_params_layout():
    # The scene-parameter dtypes mirror the C structs (sizes from the library).
    lib = N.load_scene_library()
    assert lib.bepuscene_params_size(0) == N.PILE_PARAMS_DTYPE.itemsize == 88
    assert lib.bepuscene_params_size(1) == N.TOWER_PARAMS_DTYPE.itemsize == 48
    assert lib.bepuscene_params_size(2) == N.CHAIN_PARAMS_DTYPE.itemsize
