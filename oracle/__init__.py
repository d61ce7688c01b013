"""Oracle -- test infrastructure only.

A C++ restatement of the reference's single-threaded solver path
(bepu_oracle.cpp), loaded through ctypes by the tests, the smoke check and
the CPU-baseline legs of bench.py.  Nothing in the product imports it.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .build_oracle import build as build_oracle

_lib = None

ORDER_PERMUTED, ORDER_IDENTITY = 0, 1


def _load():
    global _lib
    if _lib is None:
        from bepuphysics1_gb300 import native as N  # record dtypes only
        path = build_oracle()
        lib = ctypes.CDLL(path)
        P, I, U, F = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_float
        sig = {
            "oracle_create": (P, [P, P, I, P, I, P, I]),
            "oracle_destroy": (None, [P]),
            "oracle_set_list_order": (I, [P, P, I]),
            "oracle_set_order_mode": (None, [P, I, ctypes.c_int64]),
            "oracle_step": (I, [P, F, U, I]),
            "oracle_step_multithreaded": (I, [P, F, U, I, I]),
            "oracle_get_bodies": (None, [P, P]),
            "oracle_get_constraints": (None, [P, P, P]),
            "oracle_last_child_solves": (ctypes.c_int64, [P]),
            "oracle_permutation_map": (ctypes.c_int64, [ctypes.c_int64, ctypes.c_int64, I]),
            "oracle_prime_count": (I, []),
            "oracle_permutation_check": (ctypes.c_int64, [ctypes.c_int64, I, P]),
            "oracle_colour": (I, [P, I, P, I, P, I, P, P]),
            "oracle_set_shapes": (I, [P, P, I]),
            "oracle_set_islands": (I, [P, P, P, I, I]),
            "oracle_get_islands": (I, [P, P, I, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _ptr(a):
    if a is None or a.size == 0:
        return None
    return ctypes.c_void_p(a.ctypes.data)


def permutation_map(permutation_index: int, index: int, set_size: int) -> int:
    return _load().oracle_permutation_map(permutation_index, index, set_size)


def prime_count() -> int:
    return _load().oracle_prime_count()


def permutation_check(iterations: int, set_size: int):
    """(first permutation index that is not a permutation or -1, distinct permutations)."""
    d = ctypes.c_int64()
    k = _load().oracle_permutation_check(iterations, set_size, ctypes.byref(d))
    return k, d.value


def colour(bodies, manifolds, joints=None):
    from bepuphysics1_gb300 import native as N
    lib = _load()
    joints = np.zeros(0, N.JOINT_DTYPE) if joints is None else joints
    n = len(manifolds) + len(joints)
    col = np.zeros(n, np.int32)
    order = np.zeros(n, np.int32)
    k = lib.oracle_colour(_ptr(bodies), len(bodies), _ptr(manifolds), len(manifolds), _ptr(joints), len(joints),
                          _ptr(col), _ptr(order))
    return col, order, k


class OracleSpace:
    """The reference's Space solver stages restated on the CPU."""

    def __init__(self, settings, bodies, manifolds, joints=None, shapes=None):
        from bepuphysics1_gb300 import native as N
        self.N = N
        lib = _load()
        self.lib = lib
        self.settings = np.array(settings, dtype=N.SETTINGS_DTYPE).reshape(1)
        self.bodies = np.ascontiguousarray(bodies, dtype=N.BODY_DTYPE)
        self.manifolds = np.ascontiguousarray(manifolds, dtype=N.MANIFOLD_DTYPE)
        self.joints = np.ascontiguousarray(np.zeros(0, N.JOINT_DTYPE) if joints is None else joints,
                                           dtype=N.JOINT_DTYPE)
        h = lib.oracle_create(_ptr(self.settings), _ptr(self.bodies), len(self.bodies), _ptr(self.manifolds),
                              len(self.manifolds), _ptr(self.joints), len(self.joints))
        if not h:
            raise ValueError("oracle rejected the scene")
        self.h = ctypes.c_void_p(h)
        if shapes is not None:
            self.shapes = np.ascontiguousarray(shapes, dtype=N.SHAPE_DTYPE)
            if lib.oracle_set_shapes(self.h, _ptr(self.shapes), len(self.shapes)) != 0:
                raise ValueError("one shape per body")

    def set_list_order(self, order):
        order = np.ascontiguousarray(order, dtype=np.int32)
        if self.lib.oracle_set_list_order(self.h, _ptr(order), len(order)) != 0:
            raise ValueError("bad list order")

    def set_order_mode(self, mode: int, permutation_index: int = 0):
        self.lib.oracle_set_order_mode(self.h, mode, permutation_index)

    def step(self, dt: float, flags: int = 63, steps: int = 1):
        self.lib.oracle_step(self.h, dt, flags, steps)

    def step_multithreaded(self, dt: float, flags: int = 63, steps: int = 1, threads: int = 8):
        self.lib.oracle_step_multithreaded(self.h, dt, flags, steps, threads)

    def get_bodies(self):
        out = self.bodies.copy()
        self.lib.oracle_get_bodies(self.h, _ptr(out))
        return out

    def get_constraints(self):
        m = self.manifolds.copy()
        j = self.joints.copy()
        self.lib.oracle_get_constraints(self.h, _ptr(m), _ptr(j))
        return m, j

    def set_islands(self, island_of_body, island_flags=None, deactivation_index: int = 0):
        """The island list as bepugpu_set_islands takes it (flags default: awake,
        allowed to deactivate)."""
        from bepuphysics1_gb300 import native as N
        of = np.ascontiguousarray(island_of_body, np.int32)
        n = int(of.max(initial=-1)) + 1 if island_flags is None else len(island_flags)
        flags = (np.full(n, N.ISLAND_ACTIVE | N.ISLAND_ALLOW_DEACTIVATION, np.uint32) if island_flags is None
                 else np.ascontiguousarray(island_flags, np.uint32))
        self._island_of, self._island_flags = of, flags
        if self.lib.oracle_set_islands(self.h, _ptr(of), _ptr(flags), len(flags), int(deactivation_index)) != 0:
            raise ValueError("bad island partition")
        self.island_count = len(flags)

    def get_islands(self):
        flags = np.zeros(getattr(self, "island_count", 0), np.uint32)
        idx = ctypes.c_int32()
        if self.lib.oracle_get_islands(self.h, _ptr(flags), len(flags), ctypes.byref(idx)) != 0:
            raise ValueError("island count")
        return flags, idx.value

    def last_child_solves(self) -> int:
        return self.lib.oracle_last_child_solves(self.h)

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
