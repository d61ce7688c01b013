"""ctypes binding of the C ABI (include/bepugpu.h) and the scene source
(include/bepuscenes.h).

Records cross the boundary as numpy structured arrays whose dtypes mirror the
C structs; bepugpu_record_size() checks the layouts when the library loads.
The binding fails loudly when libbepugpu.so is missing: there is no CPU
fallback for the solver.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

LIB_DIR = Path(__file__).resolve().parent / "lib"

SETTINGS_DTYPE = np.dtype([
    ("gravity", "<f4", 3), ("iteration_limit", "<i4"), ("minimum_impulse", "<f4"),
    ("minimum_iteration_count", "<i4"), ("maximum_iteration_count", "<i4"), ("softness", "<f4"),
    ("penetration_recovery_stiffness", "<f4"), ("maximum_penetration_recovery_speed", "<f4"),
    ("static_friction_velocity_threshold", "<f4"), ("twist_friction_factor", "<f4"),
    ("bounciness_velocity_threshold", "<f4"), ("allowed_penetration", "<f4"),
    ("contact_invalidation_length_squared", "<f4"), ("maximum_contact_distance", "<f4"),
    ("use_stabilization", "<i4"), ("velocity_lower_limit", "<f4"), ("low_velocity_time_minimum", "<f4"),
    ("maximum_deactivation_attempts_per_frame", "<i4"),
])
BODY_DTYPE = np.dtype([
    ("position", "<f4", 3), ("orientation", "<f4", 4), ("linear_velocity", "<f4", 3),
    ("angular_velocity", "<f4", 3), ("inverse_mass", "<f4"), ("local_inverse_inertia", "<f4", 9),
    ("linear_damping", "<f4"), ("angular_damping", "<f4"), ("is_dynamic", "<i4"), ("activity", "<u4"),
    ("previous_velocity", "<f4"), ("velocity_time_below_limit", "<f4"),
])
CONTACT_DTYPE = np.dtype([
    ("position", "<f4", 3), ("normal", "<f4", 3), ("penetration_depth", "<f4"), ("id", "<i4"),
    ("local_offset_a", "<f4", 3), ("local_offset_b", "<f4", 3), ("base_penetration_depth", "<f4"),
    ("penetration_impulse", "<f4"), ("friction_impulse", "<f4"), ("friction_direction", "<f4", 3),
])
MANIFOLD_DTYPE = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("contact_count", "<i4"), ("flags", "<u4"),
    ("kinetic_friction", "<f4"), ("static_friction", "<f4"), ("bounciness", "<f4"),
    ("sliding_impulse", "<f4", 2), ("sliding_axis", "<f4", 3), ("twist_impulse", "<f4"), ("contact_order", "<i4"),
    ("contacts", CONTACT_DTYPE, 4),
])
BODY_STATE_DTYPE = np.dtype([
    ("position", "<f4", 3), ("orientation", "<f4", 4), ("linear_velocity", "<f4", 3),
    ("angular_velocity", "<f4", 3), ("activity", "<u4"), ("previous_velocity", "<f4"),
    ("velocity_time_below_limit", "<f4"),
])
MANIFOLD_STATE_DTYPE = np.dtype([
    ("contact_count", "<i4"), ("contact_id", "<i4", 4), ("penetration_impulse", "<f4", 4),
    ("sliding_impulse", "<f4", 2), ("twist_impulse", "<f4"), ("sliding_axis", "<f4", 3),
    ("friction_impulse", "<f4", 4), ("reserved", "<i4"),
])
SHAPE_DTYPE = np.dtype([("type", "<i4"), ("size", "<f4", 3)])
JOINT_DTYPE = np.dtype([
    ("type", "<i4"), ("body_a", "<i4"), ("body_b", "<i4"), ("flags", "<u4"),
    ("anchor_a", "<f4", 3), ("anchor_b", "<f4", 3), ("axis_a", "<f4", 3), ("axis_b", "<f4", 3),
    ("constrained_1", "<f4", 3), ("constrained_2", "<f4", 3), ("basis_primary", "<f4", 3), ("basis_x", "<f4", 3),
    ("test_axis", "<f4", 3), ("limit_min", "<f4"), ("limit_max", "<f4"), ("margin", "<f4"), ("bounciness", "<f4"),
    ("bounce_velocity_threshold", "<f4"), ("max_corrective_velocity", "<f4"), ("spring_stiffness", "<f4"),
    ("spring_damping", "<f4"), ("impulse", "<f4", 8), ("orientation_a", "<f4", 4), ("orientation_b", "<f4", 4),
])

PILE_PARAMS_DTYPE = np.dtype([
    ("nx", "<i4"), ("ny", "<i4"), ("nz", "<i4"), ("spacing", "<f4"), ("size_min", "<f4"), ("size_max", "<f4"),
    ("density", "<f4"), ("mass", "<f4"), ("jitter", "<f4"), ("friction_min", "<f4"), ("friction_max", "<f4"),
    ("ground_friction", "<f4"), ("ground_size", "<f4", 3), ("settle_penetration", "<f4"),
    ("contact_distance", "<f4"), ("seed", "<u8"), ("narrow_phase", "<i4"), ("drop_spacing", "<f4"),
], align=True)
TOWER_PARAMS_DTYPE = np.dtype([
    ("body_count", "<i4"), ("tower_min", "<i4"), ("tower_max", "<i4"), ("sphere_fraction", "<f4"),
    ("friction", "<f4"), ("tower_spacing", "<f4"), ("settle_penetration", "<f4"), ("seed", "<u8"),
    ("narrow_phase", "<i4"),
], align=True)
CHAIN_PARAMS_DTYPE = np.dtype([
    ("chains", "<i4"), ("links", "<i4"), ("capsule_radius", "<f4"), ("capsule_length", "<f4"),
    ("link_mass", "<f4"), ("swing_limit", "<f4"), ("loose_bodies", "<i4"), ("region", "<f4", 3),
    ("seed", "<u8"),
], align=True)

SERVER_CONFIG_DTYPE = np.dtype([
    ("device_budget_bytes", "<u8"), ("max_wave_scenes", "<u4"), ("max_waves_in_flight", "<u4"),
    ("queue_capacity", "<u4"), ("batching", "<u4"), ("dt", "<f4"), ("flags", "<u4"), ("threads", "<u4"),
    ("reserved", "<u4", 3),
])
COMPLETION_DTYPE = np.dtype([
    ("tag", "<u8"), ("scene", "<i4"), ("status", "<i4"), ("steps", "<u4"), ("wave", "<u4"),
    ("submit_us", "<f8"), ("start_us", "<f8"), ("done_us", "<f8"),
])
SERVER_STATS_DTYPE = np.dtype([
    ("submitted", "<u8"), ("completed", "<u8"), ("waves", "<u8"), ("wave_scenes", "<u8"), ("launches", "<u8"),
    ("spills", "<u8"), ("restores", "<u8"), ("resident_bytes", "<u8"), ("peak_resident_bytes", "<u8"),
    ("spilled_bytes", "<u8"), ("scenes", "<u4"), ("resident_scenes", "<u4"), ("room_waits", "<u8"),
    ("restore_failures", "<u8"), ("spill_us", "<u8"), ("restore_us", "<u8"), ("pinned_bytes", "<u8"),
])

PHASE_TIMES_DTYPE = np.dtype([
    ("refresh_ms", "<f4"), ("force_ms", "<f4"), ("prestep_ms", "<f4"), ("warm_ms", "<f4"), ("solve_ms", "<f4"),
    ("position_ms", "<f4"), ("solve_launches", "<u4"), ("warm_launches", "<u4"),
    ("solve_algorithmic_bytes", "<f8"), ("solve_manifold_visits", "<f8"), ("solve_contact_visits", "<f8"),
    ("group_ms", "<f4"), ("groups", "<u4"), ("group_compulsory_bytes", "<f8"),
    ("group_solve_algorithmic_bytes", "<f8"), ("group_solve_manifold_visits", "<f8"),
])

# bepugpu_status
OK, INVALID_ARGUMENT, OUT_OF_MEMORY, ADMISSION_REFUSED, CUDA_ERROR, TIMEOUT, NAN_DETECTED, NOT_FOUND, \
    QUEUE_FULL, INVALID_OPERATION = range(10)
STATUS_NAMES = ["OK", "INVALID_ARGUMENT", "OUT_OF_MEMORY", "ADMISSION_REFUSED", "CUDA_ERROR", "TIMEOUT",
                "NAN_DETECTED", "NOT_FOUND", "QUEUE_FULL", "INVALID_OPERATION"]

STEP_REFRESH_CONTACTS, STEP_FORCES, STEP_SOLVE, STEP_POSITIONS, STEP_COLLIDE = 1, 2, 4, 8, 16
STEP_DEACTIVATION, STEP_ALL = 32, 63
BODY_ALWAYS_ACTIVE, BODY_NO_STABILIZATION, BODY_SLOWING, BODY_DEACTIVATION_CANDIDATE = 1, 2, 4, 8
SHAPE_NONE, SHAPE_BOX, SHAPE_SPHERE = 0, 1, 2
NOALLOC_MAX_BODIES, NOALLOC_MAX_MANIFOLDS = 1024, 2048  # bepugpu_step_noalloc limits
MODE_GRAPH, MODE_PERSISTENT = 0, 1
MANIFOLD_ACTIVE, MANIFOLD_SOLVER_RULE, MANIFOLD_GENERATED, MANIFOLD_NONCONVEX = 1, 2, 4, 8
JOINT_BALL_SOCKET, JOINT_REVOLUTE_ANGULAR, JOINT_SWING_LIMIT, JOINT_REVOLUTE_LIMIT, JOINT_REVOLUTE = 1, 2, 3, 4, 5
JOINT_NO_ROTATION, JOINT_WELD, JOINT_DISTANCE, JOINT_DISTANCE_LIMIT = 6, 7, 8, 9
JOINT_POINT_ON_PLANE, JOINT_TWIST = 10, 11
JOINT_POINT_ON_LINE, JOINT_PRISMATIC, JOINT_LINE_SLIDER, JOINT_UNIVERSAL = 12, 13, 14, 15
JOINT_TWIST_LIMIT, JOINT_LINEAR_AXIS_LIMIT, JOINT_ELLIPSE_SWING_LIMIT = 16, 17, 18
JOINT_SWIVEL_HINGE_ANGULAR, JOINT_SWIVEL_HINGE = 19, 20
JOINT_REVOLUTE_MOTOR, JOINT_TWIST_MOTOR, JOINT_LINEAR_AXIS_MOTOR = 21, 22, 23
JOINT_MAXIMUM_LINEAR_SPEED, JOINT_MAXIMUM_ANGULAR_SPEED, JOINT_PLANE_SLIDER = 24, 25, 26
JOINT_ANGULAR_MOTOR, JOINT_SINGLE_ENTITY_ANGULAR_MOTOR, JOINT_SINGLE_ENTITY_LINEAR_MOTOR = 27, 28, 29
JOINT_ACTIVE, JOINT_LIMIT_ACTIVE, JOINT_SERVO, JOINT_GROUP_CONTINUATION = 1, 2, 4, 8
ISLAND_ACTIVE, ISLAND_ALLOW_DEACTIVATION = 1, 2

_P = ctypes.c_void_p
_I = ctypes.c_int32
_U = ctypes.c_uint32
_F = ctypes.c_float

# name: (restype, argtypes)
GPU_EXPORTS = {
    "bepugpu_probe_double_rounding": (_I, [_P, _I, _P, _P, _U, _P, _P]),
    "bepugpu_abi_version": (_I, []),
    "bepugpu_record_size": (_U, [_I]),
    "bepugpu_default_settings": (None, [_P]),
    "bepugpu_create": (_I, [_I, _P, ctypes.POINTER(_P)]),
    "bepugpu_destroy": (None, [_P]),
    "bepugpu_last_error": (ctypes.c_char_p, [_P]),
    "bepugpu_set_settings": (_I, [_P, _P]),
    "bepugpu_synchronize": (_I, [_P]),
    "bepugpu_memory_usage": (_I, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "bepugpu_scene_create": (_I, [_P, _U, _U, _U, ctypes.POINTER(_I)]),
    "bepugpu_scene_destroy": (_I, [_P, _I]),
    "bepugpu_upload_bodies": (_I, [_P, _I, _P, _U]),
    "bepugpu_upload_shapes": (_I, [_P, _I, _P, _U]),
    "bepugpu_broad_phase": (_I, [_P, _I, _F, _P, _U, ctypes.POINTER(_U)]),
    "bepugpu_set_islands": (_I, [_P, _I, _P, _U, _P, _U, _I]),
    "bepugpu_set_materials": (_I, [_P, _I, _P, _U]),
    "bepugpu_update_pairs": (_I, [_P, _I, _F, ctypes.POINTER(_U)]),
    "bepugpu_get_islands": (_I, [_P, _I, _P, _U, ctypes.POINTER(_I)]),
    "bepugpu_step_host": (_I, [_P, _I, _P, _U, _P, _U, ctypes.c_float, _U]),
    "bepugpu_step_state": (_I, [_P, _I, _P, _U, _P, _U, ctypes.c_float, _U]),
    "bepugpu_download_state": (_I, [_P, _I, _P, _U, _P, _U]),
    "bepugpu_upload_constraints": (_I, [_P, _I, _P, _U, _P, _U]),
    "bepugpu_update_manifolds": (_I, [_P, _I, _P, _U]),
    "bepugpu_update_bodies": (_I, [_P, _I, _P, _U]),
    "bepugpu_check_finite": (_I, [_P, _I, ctypes.POINTER(_I)]),
    "bepugpu_probe_bounded_wait": (_I, [_P, _U]),
    "bepugpu_download_bodies": (_I, [_P, _I, _P, _U]),
    "bepugpu_download_constraints": (_I, [_P, _I, _P, _U, _P, _U]),
    "bepugpu_get_colouring": (_I, [_P, _I, _P, _P, _U, ctypes.POINTER(_U)]),
    "bepugpu_colour_list": (_I, [_P, _P, _U, _P, _U, _P, _P, ctypes.POINTER(_U)]),
    "bepugpu_step": (_I, [_P, _I, _F, _U]),
    "bepugpu_set_solve_mode": (_I, [_P, _I, _I]),
    "bepugpu_set_persistent_blocks_per_sm": (_I, [_P, _I, _I]),
    "bepugpu_set_group_policy": (_I, [_P, _I, _I, _I, _I, _I, _I]),
    "bepugpu_set_group_smem_budget": (_I, [_P, _I, _U]),
    "bepugpu_set_group_prologue": (_I, [_P, _I, _I]),
    "bepugpu_set_batch_threads": (_I, [_P, _I]),
    "bepugpu_last_step_ms": (_I, [_P, _I, ctypes.POINTER(_F)]),
    "bepugpu_last_step_launches": (_I, [_P, _I, ctypes.POINTER(_U)]),
    "bepugpu_last_step_phase_ms": (_I, [_P, _I, _P]),
    "bepugpu_batch_step": (_I, [_P, _P, _U, _F, _U, _U]),
    "bepugpu_batch_step_each": (_I, [_P, _P, _P, _U, _F, _U]),
    "bepugpu_profile_step": (_I, [_P, _I, _F, _U, _P]),
    "bepugpu_step_noalloc": (_I, [_P, _P, _U, _P, _U, _F, _U, _P]),
    "bepugpu_last_call_stats": (_I, [_P, ctypes.POINTER(_U), ctypes.POINTER(_F)]),
    "bepugpu_server_default_config": (None, [_P]),
    "bepugpu_server_create": (_I, [_P, _P, ctypes.POINTER(_P)]),
    "bepugpu_server_destroy": (_I, [_P]),
    "bepugpu_server_add_scene": (_I, [_P, _I]),
    "bepugpu_server_release_scene": (_I, [_P, _I, _U]),
    "bepugpu_serve_submit": (_I, [_P, _I, _U, ctypes.c_uint64]),
    "bepugpu_serve_poll": (_I, [_P, _P, _U, ctypes.POINTER(_U)]),
    "bepugpu_server_drain": (_I, [_P, _U]),
    "bepugpu_server_stats_get": (_I, [_P, _P]),
    "bepugpu_server_last_error": (ctypes.c_char_p, [_P]),
    "bepugpu_clock_us": (ctypes.c_double, []),
}

SCENE_EXPORTS = {
    "bepuscene_default_pile": (None, [_P]),
    "bepuscene_default_tower": (None, [_P]),
    "bepuscene_default_chain": (None, [_P]),
    "bepuscene_make_pile": (_I, [_P, ctypes.POINTER(_P)]),
    "bepuscene_make_tower": (_I, [_P, ctypes.POINTER(_P)]),
    "bepuscene_make_chain": (_I, [_P, ctypes.POINTER(_P)]),
    "bepuscene_counts": (None, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "bepuscene_copy": (None, [_P, _P, _P, _P]),
    "bepuscene_shapes": (None, [_P, _P]),
    "bepuscene_body_friction": (None, [_P, _P]),
    "bepuscene_params_size": (_U, [_I]),
    "bepuscene_free": (None, [_P]),
}

_gpu = None
_scenes = None


def _bind(lib, table):
    for name, (res, args) in table.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def load_gpu_library(path: str | None = None):
    """Loads libbepugpu.so (raises when it has not been built)."""
    global _gpu
    if _gpu is not None and path is None:
        return _gpu
    p = Path(path) if path else LIB_DIR / "libbepugpu.so"
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with __graft_entry__.build() "
                           "(the solver has no CPU fallback)")
    lib = _bind(ctypes.CDLL(str(p)), GPU_EXPORTS)
    sizes = {0: SETTINGS_DTYPE, 1: BODY_DTYPE, 2: CONTACT_DTYPE, 3: MANIFOLD_DTYPE, 4: JOINT_DTYPE,
             5: BODY_STATE_DTYPE, 6: MANIFOLD_STATE_DTYPE}
    for kind, dt in sizes.items():
        got = lib.bepugpu_record_size(kind)
        if got != dt.itemsize:
            raise RuntimeError(f"record {kind}: library size {got} != binding size {dt.itemsize}")
    if path is None:
        _gpu = lib
    return lib


def load_scene_library():
    global _scenes
    if _scenes is None:
        p = LIB_DIR / "libbepuscenes.so"
        if not p.exists():
            raise RuntimeError(f"{p} is missing: build it with __graft_entry__.build()")
        _scenes = _bind(ctypes.CDLL(str(p)), SCENE_EXPORTS)
    return _scenes


def ptr(a: np.ndarray | None):
    if a is None or a.size == 0:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


class BepuError(RuntimeError):
    """A failing C-ABI call: carries the status code and the library's message."""

    def __init__(self, status: int, message: str):
        self.status = status
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{name}: {message}")


class ArgumentException(BepuError, ValueError):
    """Raised for BEPUGPU_INVALID_ARGUMENT, as the reference throws ArgumentException."""


class InvalidOperationException(BepuError):
    """Raised for BEPUGPU_INVALID_OPERATION (the reference's InvalidOperationException)."""


def raise_for(status: int, message: str):
    if status == OK:
        return
    if status in (INVALID_ARGUMENT, NOT_FOUND):
        raise ArgumentException(status, message)
    if status == INVALID_OPERATION:
        raise InvalidOperationException(status, message)
    raise BepuError(status, message)
