"""Shared helpers of the GPU parity tests: run the device solver and the
oracle's colour-order restatement side by side and compare."""
from __future__ import annotations

import numpy as np

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300.solver import GpuSpace, default_settings

DT = np.float32(1 / 60)

# Tolerances of the parity bar: FP32 per-body linear/angular velocities and
# accumulated impulses agree to <= 1e-4 relative after each step and <= 1e-3
# after 60 steps.  "Relative" is max |gpu - oracle| over an array divided by
# max |oracle| over the same array.
STEP_TOL = 1e-4
LONG_TOL = 1e-3


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(initial=0.0), 1e-12)
    return float(np.abs(a - b).max(initial=0.0) / scale)


def compare(gb, gm, ob, om, gj=None, oj=None):
    """Relative errors of velocities, positions and impulses; the contact
    counts and indexing must agree exactly."""
    np.testing.assert_array_equal(gm["contact_count"], om["contact_count"])
    np.testing.assert_array_equal(gm["contacts"]["id"], om["contacts"]["id"])
    errs = {
        "linear_velocity": rel_err(gb["linear_velocity"], ob["linear_velocity"]),
        "angular_velocity": rel_err(gb["angular_velocity"], ob["angular_velocity"]),
        "position": rel_err(gb["position"], ob["position"]),
        "orientation": rel_err(gb["orientation"], ob["orientation"]),
        "penetration_impulse": rel_err(gm["contacts"]["penetration_impulse"], om["contacts"]["penetration_impulse"]),
        "sliding_impulse": rel_err(gm["sliding_impulse"], om["sliding_impulse"]),
        "twist_impulse": rel_err(gm["twist_impulse"], om["twist_impulse"]),
    }
    exact = (np.array_equal(gb["linear_velocity"], ob["linear_velocity"]) and
             np.array_equal(gb["angular_velocity"], ob["angular_velocity"]) and
             np.array_equal(gm["contacts"]["penetration_impulse"], om["contacts"]["penetration_impulse"]))
    if gj is not None and len(gj):
        errs["joint_impulse"] = rel_err(gj["impulse"], oj["impulse"])
        exact = exact and np.array_equal(gj["impulse"], oj["impulse"])
    return errs, exact


class Pair:
    """A GPU scene and the oracle over the same records, the oracle's solver
    list permuted into the GPU's colour order (identity mapping)."""

    def __init__(self, ctx, bodies, manifolds, joints=None, settings=None, mode=N.MODE_GRAPH, group_policy=None,
                 shapes=None):
        self.joints = joints
        self.settings = default_settings() if settings is None else settings
        ctx.set_settings(self.settings)
        self.gpu = GpuSpace(ctx, bodies, manifolds, joints, group_policy=group_policy, shapes=shapes)
        self.gpu.set_mode(mode)
        colour, order, k = self.gpu.colouring()
        self.colours = k
        self.order = order
        self.oracle = oracle.OracleSpace(self.settings, bodies, manifolds, joints, shapes=shapes)
        self.oracle.set_list_order(order)
        self.oracle.set_order_mode(oracle.ORDER_IDENTITY)

    def step(self, flags=N.STEP_ALL, steps=1, dt=DT):
        for _ in range(steps):
            self.gpu.step(dt, flags)
        self.oracle.step(dt, flags, steps)

    def compare(self):
        gb = self.gpu.download_bodies()
        gj0 = None if self.joints is None else self.joints.copy()
        gm, gj = self.gpu.download_constraints(joints=gj0)
        ob = self.oracle.get_bodies()
        om, oj = self.oracle.get_constraints()
        return compare(gb, gm, ob, om, gj, oj)

    def close(self):
        self.gpu.close()
        self.oracle.close()
