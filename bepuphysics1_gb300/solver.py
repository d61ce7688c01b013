"""Host-side mirror of the reference's solver-stage surface over the C ABI.

The reference hands its solver stage a list of SolverUpdateables and calls
    Solver.Update()            (Constraints/Solver.cs:239-263)
    ForceUpdater.Update()      (OtherSpaceStages/ForceUpdater.cs:73-92)
    PositionUpdater.Update()   (PositionUpdating/ContinuousPositionUpdater.cs:134-154)
once per Space.Update (Space.cs:496-522).  `GpuSpace` keeps one scene resident
on the device and exposes the same stages; `Solver.iteration_limit` mirrors
Solver.IterationLimit (Solver.cs:15-19, clamped at zero like the property).
Errors come back as ArgumentException / InvalidOperationException like the
reference's.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native as N


class Context:
    """One device and the reference's global settings (bepugpu_settings)."""

    def __init__(self, device: int = 0, settings: np.ndarray | None = None):
        self.lib = N.load_gpu_library()
        if settings is None:
            settings = default_settings()
        self.settings = np.array(settings, dtype=N.SETTINGS_DTYPE).reshape(())
        h = ctypes.c_void_p()
        st = self.lib.bepugpu_create(device, N.ptr(self.settings.reshape(1)), ctypes.byref(h))
        if st != N.OK:
            N.raise_for(st, f"bepugpu_create(device={device}) failed")
        self.handle = h

    def check(self, status: int):
        if status != N.OK:
            msg = self.lib.bepugpu_last_error(self.handle)
            N.raise_for(status, msg.decode() if msg else "")

    def set_settings(self, settings: np.ndarray):
        self.settings = np.array(settings, dtype=N.SETTINGS_DTYPE).reshape(())
        self.check(self.lib.bepugpu_set_settings(self.handle, N.ptr(self.settings.reshape(1))))

    def synchronize(self):
        self.check(self.lib.bepugpu_synchronize(self.handle))

    def memory_usage(self) -> tuple[int, int]:
        """(reserved, in_use) bytes of the device heap that holds scene arenas."""
        r, u = ctypes.c_uint64(), ctypes.c_uint64()
        self.check(self.lib.bepugpu_memory_usage(self.handle, ctypes.byref(r), ctypes.byref(u)))
        return r.value, u.value

    def close(self):
        if getattr(self, "handle", None):
            self.lib.bepugpu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_settings() -> np.ndarray:
    lib = N.load_gpu_library()
    s = np.zeros(1, dtype=N.SETTINGS_DTYPE)
    lib.bepugpu_default_settings(N.ptr(s))
    return s[0].copy()


class Solver:
    """Mirror of Solver's settable surface for one scene."""

    def __init__(self, space: "GpuSpace"):
        self._space = space

    @property
    def iteration_limit(self) -> int:
        return int(self._space.ctx.settings["iteration_limit"])

    @iteration_limit.setter
    def iteration_limit(self, value: int):
        s = self._space.ctx.settings.copy()
        s["iteration_limit"] = max(int(value), 0)
        self._space.ctx.set_settings(s)

    def update(self, dt: float):
        """Solver.Update: prestep, warm start and iterations."""
        self._space.step(dt, N.STEP_SOLVE)


class GpuSpace:
    """One scene resident on the device: bodies plus the solver list."""

    def __init__(self, ctx: Context, bodies: np.ndarray, manifolds: np.ndarray | None = None,
                 joints: np.ndarray | None = None, capacity: tuple[int, int, int] | None = None,
                 group_policy: tuple[int, int, int, int, int] | None = None, smem_budget: int | None = None,
                 shapes: np.ndarray | None = None):
        """group_policy = (enabled, max_bodies, max_manifolds, target_manifolds, threads),
        see bepugpu_set_group_policy; smem_budget = bepugpu_set_group_smem_budget;
        None keeps the library defaults.  shapes: one bepugpu_shape per body,
        needed by GENERATED manifolds (uploaded before the constraints)."""
        self.ctx = ctx
        lib = ctx.lib
        manifolds = np.zeros(0, N.MANIFOLD_DTYPE) if manifolds is None else manifolds
        joints = np.zeros(0, N.JOINT_DTYPE) if joints is None else joints
        cap = capacity or (len(bodies), len(manifolds), len(joints))
        sid = ctypes.c_int32()
        ctx.check(lib.bepugpu_scene_create(ctx.handle, cap[0], cap[1], cap[2], ctypes.byref(sid)))
        self.id = sid.value
        self.solver = Solver(self)
        if group_policy is not None:
            self.set_group_policy(*group_policy)
        if smem_budget is not None:
            self.set_group_smem_budget(smem_budget)
        self.upload_bodies(bodies)
        if shapes is not None:
            self.upload_shapes(shapes)
        self.upload_constraints(manifolds, joints)

    def upload_shapes(self, shapes: np.ndarray):
        """bepugpu_upload_shapes: one collision shape per body for the narrow phase."""
        shapes = np.ascontiguousarray(shapes, dtype=N.SHAPE_DTYPE)
        self.ctx.check(self.ctx.lib.bepugpu_upload_shapes(self.ctx.handle, self.id, N.ptr(shapes), len(shapes)))

    def set_group_policy(self, enabled: int = 1, max_bodies: int = 1024, max_manifolds: int = 4096,
                         target_manifolds: int = 64, threads: int = 0):
        self.ctx.check(self.ctx.lib.bepugpu_set_group_policy(self.ctx.handle, self.id, enabled, max_bodies,
                                                             max_manifolds, target_manifolds, threads))

    def set_group_smem_budget(self, nbytes: int):
        """bepugpu_set_group_smem_budget: groups needing more shared memory keep
        their solve lanes in global memory (next upload_constraints)."""
        self.ctx.check(self.ctx.lib.bepugpu_set_group_smem_budget(self.ctx.handle, self.id, int(nbytes)))

    def set_group_prologue(self, mode: int):
        """bepugpu_set_group_prologue: the island groups' refresh, body updates
        and prestep inside the group kernel (0), as grid-wide launches before
        it (1), or by scene size (-1, the default)."""
        self.ctx.check(self.ctx.lib.bepugpu_set_group_prologue(self.ctx.handle, self.id, int(mode)))

    def upload_bodies(self, bodies: np.ndarray):
        bodies = np.ascontiguousarray(bodies, dtype=N.BODY_DTYPE)
        self.ctx.check(self.ctx.lib.bepugpu_upload_bodies(self.ctx.handle, self.id, N.ptr(bodies), len(bodies)))
        self.body_count = len(bodies)

    def upload_constraints(self, manifolds: np.ndarray, joints: np.ndarray | None = None):
        manifolds = np.ascontiguousarray(manifolds, dtype=N.MANIFOLD_DTYPE)
        joints = np.ascontiguousarray(np.zeros(0, N.JOINT_DTYPE) if joints is None else joints, dtype=N.JOINT_DTYPE)
        self.ctx.check(self.ctx.lib.bepugpu_upload_constraints(
            self.ctx.handle, self.id, N.ptr(manifolds), len(manifolds), N.ptr(joints), len(joints)))
        self.manifold_count = len(manifolds)
        self.joint_count = len(joints)

    def set_materials(self, materials: np.ndarray):
        """bepugpu_set_materials: per body (kinetic friction, static friction,
        bounciness), blended by product into new pairs' records."""
        mat = np.ascontiguousarray(materials, np.float32).reshape(-1, 3)
        self.ctx.check(self.ctx.lib.bepugpu_set_materials(self.ctx.handle, self.id, N.ptr(mat), len(mat)))

    def update_pairs(self, dt: float) -> int:
        """bepugpu_update_pairs: the manifold list follows the broad phase's pair
        set on the device (new GENERATED records, ended pairs dropped, recoloured).
        Returns the new manifold count."""
        n = ctypes.c_uint32()
        self.ctx.check(self.ctx.lib.bepugpu_update_pairs(self.ctx.handle, self.id, float(dt), ctypes.byref(n)))
        self.manifold_count = n.value
        return n.value

    def update_bodies(self, bodies: np.ndarray):
        """bepugpu_update_bodies: new position, orientation and velocities only."""
        bodies = np.ascontiguousarray(bodies, dtype=N.BODY_DTYPE)
        self.ctx.check(self.ctx.lib.bepugpu_update_bodies(self.ctx.handle, self.id, N.ptr(bodies), len(bodies)))

    def update_manifolds(self, manifolds: np.ndarray):
        manifolds = np.ascontiguousarray(manifolds, dtype=N.MANIFOLD_DTYPE)
        self.ctx.check(self.ctx.lib.bepugpu_update_manifolds(self.ctx.handle, self.id, N.ptr(manifolds),
                                                             len(manifolds)))

    def step_host(self, bodies: np.ndarray, manifolds: np.ndarray, dt: float, flags: int = N.STEP_ALL):
        """bepugpu_step_host: new body state and manifold records up, one step,
        whole records back into the same (ideally pinned) arrays."""
        assert bodies.dtype == N.BODY_DTYPE and manifolds.dtype == N.MANIFOLD_DTYPE
        assert bodies.flags.c_contiguous and manifolds.flags.c_contiguous
        self.ctx.check(self.ctx.lib.bepugpu_step_host(self.ctx.handle, self.id, N.ptr(bodies), len(bodies),
                                                      N.ptr(manifolds), len(manifolds), float(dt), flags))

    def step_state(self, bodies: np.ndarray, manifolds: np.ndarray | None, dt: float, flags: int = N.STEP_ALL):
        """bepugpu_step_state: body state up, one step, body state back into
        `bodies` and the manifolds' impulses into `manifolds` (None: skipped)."""
        assert bodies.dtype == N.BODY_STATE_DTYPE and bodies.flags.c_contiguous
        nm = 0
        if manifolds is not None:
            assert manifolds.dtype == N.MANIFOLD_STATE_DTYPE and manifolds.flags.c_contiguous
            nm = len(manifolds)
        self.ctx.check(self.ctx.lib.bepugpu_step_state(self.ctx.handle, self.id, N.ptr(bodies), len(bodies),
                                                       N.ptr(manifolds), nm, float(dt), flags))

    def broad_phase(self, dt: float, max_pairs: int | None = None) -> np.ndarray:
        """bepugpu_broad_phase: the overlapping pairs of shaped bodies as an
        (n, 2) int32 array, ascending; grows the buffer once when max_pairs is
        too small (None: start at four pairs a body)."""
        cap = 4 * self.body_count if max_pairs is None else max_pairs
        for _ in range(2):
            out = np.zeros((max(cap, 1), 2), np.int32)
            n = ctypes.c_uint32()
            self.ctx.check(self.ctx.lib.bepugpu_broad_phase(self.ctx.handle, self.id, float(dt), N.ptr(out), cap,
                                                            ctypes.byref(n)))
            if n.value <= cap:
                return out[:n.value]
            cap = n.value
        raise RuntimeError("broad phase pair count kept growing")

    def download_state(self, bodies: np.ndarray | None = None, manifolds: np.ndarray | None = None):
        """bepugpu_download_state into the given state arrays (either may be None)."""
        nb = 0 if bodies is None else len(bodies)
        nm = 0 if manifolds is None else len(manifolds)
        assert bodies is None or bodies.dtype == N.BODY_STATE_DTYPE
        assert manifolds is None or manifolds.dtype == N.MANIFOLD_STATE_DTYPE
        self.ctx.check(self.ctx.lib.bepugpu_download_state(self.ctx.handle, self.id, N.ptr(bodies), nb,
                                                           N.ptr(manifolds), nm))
        return bodies, manifolds

    def set_mode(self, mode: int):
        self.ctx.check(self.ctx.lib.bepugpu_set_solve_mode(self.ctx.handle, self.id, mode))

    def step(self, dt: float, flags: int = N.STEP_ALL):
        """Space.Update's velocity and integration stages in pipeline order."""
        self.ctx.check(self.ctx.lib.bepugpu_step(self.ctx.handle, self.id, float(dt), flags))

    def deactivation_update(self, dt: float):
        """DeactivationManager.Update's per-member part: every body's
        UpdateDeactivationCandidacy (SimulationIslandMember.cs:53-164)."""
        self.step(dt, N.STEP_DEACTIVATION)

    def force_update(self, dt: float):
        self.step(dt, N.STEP_FORCES)

    def position_update(self, dt: float):
        self.step(dt, N.STEP_POSITIONS)

    def refresh_contacts(self, dt: float):
        self.step(dt, N.STEP_REFRESH_CONTACTS)

    def set_islands(self, island_of_body: np.ndarray, island_flags: np.ndarray | None = None,
                    deactivation_index: int = 0):
        """bepugpu_set_islands: the island list (one entry per island, BEPUGPU_ISLAND_*
        flags; default awake and allowed to deactivate) and each body's island
        (-1 for kinematic bodies)."""
        of = np.ascontiguousarray(island_of_body, np.int32)
        n = int(of.max(initial=-1)) + 1 if island_flags is None else len(island_flags)
        flags = (np.full(n, N.ISLAND_ACTIVE | N.ISLAND_ALLOW_DEACTIVATION, np.uint32) if island_flags is None
                 else np.ascontiguousarray(island_flags, np.uint32))
        self.ctx.check(self.ctx.lib.bepugpu_set_islands(self.ctx.handle, self.id, N.ptr(of), len(of), N.ptr(flags),
                                                        len(flags), int(deactivation_index)))
        self.island_count = len(flags)

    def get_islands(self):
        """(island flags, deactivation index) as the last step left them."""
        flags = np.zeros(getattr(self, "island_count", 0), np.uint32)
        idx = ctypes.c_int32()
        self.ctx.check(self.ctx.lib.bepugpu_get_islands(self.ctx.handle, self.id, N.ptr(flags), len(flags),
                                                        ctypes.byref(idx)))
        return flags, idx.value

    def download_bodies(self, into: np.ndarray | None = None) -> np.ndarray:
        out = np.zeros(self.body_count, N.BODY_DTYPE) if into is None else into
        self.ctx.check(self.ctx.lib.bepugpu_download_bodies(self.ctx.handle, self.id, N.ptr(out), len(out)))
        return out

    def download_constraints(self, manifolds: np.ndarray | None = None, joints: np.ndarray | None = None):
        m = np.zeros(self.manifold_count, N.MANIFOLD_DTYPE) if manifolds is None else manifolds
        j = np.zeros(self.joint_count, N.JOINT_DTYPE) if joints is None else joints
        self.ctx.check(self.ctx.lib.bepugpu_download_constraints(self.ctx.handle, self.id, N.ptr(m), len(m),
                                                                 N.ptr(j), len(j)))
        return m, j

    def colouring(self):
        n = self.manifold_count + self.joint_count
        colour = np.zeros(n, np.int32)
        order = np.zeros(n, np.int32)
        k = ctypes.c_uint32()
        self.ctx.check(self.ctx.lib.bepugpu_get_colouring(self.ctx.handle, self.id, N.ptr(colour), N.ptr(order), n,
                                                          ctypes.byref(k)))
        return colour, order, k.value

    def check_finite(self) -> int:
        """bepugpu_check_finite: -1, or raises BepuError(NAN_DETECTED) naming the
        first body with a non-finite state."""
        bad = ctypes.c_int32()
        self.ctx.check(self.ctx.lib.bepugpu_check_finite(self.ctx.handle, self.id, ctypes.byref(bad)))
        return bad.value

    def last_step_ms(self) -> float:
        v = ctypes.c_float()
        self.ctx.check(self.ctx.lib.bepugpu_last_step_ms(self.ctx.handle, self.id, ctypes.byref(v)))
        return v.value

    def last_step_phase_ms(self) -> np.ndarray:
        """[refresh + forces, prestep, warm start, solve, positions, island groups] device ms."""
        out = np.zeros(6, np.float32)
        self.ctx.check(self.ctx.lib.bepugpu_last_step_phase_ms(self.ctx.handle, self.id, N.ptr(out)))
        return out

    def last_step_launches(self) -> int:
        v = ctypes.c_uint32()
        self.ctx.check(self.ctx.lib.bepugpu_last_step_launches(self.ctx.handle, self.id, ctypes.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "id", None) is not None and self.ctx.handle:
            self.ctx.lib.bepugpu_scene_destroy(self.ctx.handle, self.id)
            self.id = None


def body_states(bodies: np.ndarray, out: np.ndarray | None = None) -> np.ndarray:
    """The state fields of body records as bepugpu_body_state records."""
    if out is None:
        out = np.zeros(len(bodies), N.BODY_STATE_DTYPE)
    for f in N.BODY_STATE_DTYPE.names:
        out[f] = bodies[f]
    return out


def colour_list(bodies: np.ndarray, manifolds: np.ndarray, joints: np.ndarray | None = None):
    """The library's colouring of a solver list (joints first, then manifolds),
    computed on the host: (colour per updateable, colour-sorted order, colours)."""
    lib = N.load_gpu_library()
    joints = np.zeros(0, N.JOINT_DTYPE) if joints is None else joints
    a = np.ascontiguousarray(np.concatenate([joints["body_a"], manifolds["body_a"]]).astype(np.int32))
    b = np.ascontiguousarray(np.concatenate([joints["body_b"], manifolds["body_b"]]).astype(np.int32))
    dyn = np.ascontiguousarray((bodies["is_dynamic"] != 0).astype(np.uint8))
    n = len(a)
    colour = np.zeros(n, np.int32)
    order = np.zeros(n, np.int32)
    k = ctypes.c_uint32()
    st = lib.bepugpu_colour_list(N.ptr(a), N.ptr(b), n, N.ptr(dyn), len(dyn), N.ptr(colour), N.ptr(order),
                                 ctypes.byref(k))
    N.raise_for(st, "bepugpu_colour_list: a constraint references a body outside the body array")
    return colour, order, k.value


def islands_of(bodies: np.ndarray, manifolds: np.ndarray, joints: np.ndarray | None = None) -> np.ndarray:
    """A partition for bepugpu_set_islands when no DeactivationManager keeps one:
    dynamic bodies joined through every joint and every manifold with contacts
    (the SimulationIslandConnections of the constraints in the solver),
    islands numbered in the order of their first member.  -1 for kinematic
    bodies."""
    nb = len(bodies)
    parent = np.arange(nb)

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    dyn = bodies["is_dynamic"] != 0
    pairs = []
    if joints is not None and len(joints):
        pairs.append(np.stack([joints["body_a"], joints["body_b"]], 1))
    if len(manifolds):
        has = manifolds["contact_count"] > 0
        pairs.append(np.stack([manifolds["body_a"][has], manifolds["body_b"][has]], 1))
    for a, b in (np.concatenate(pairs) if pairs else np.zeros((0, 2), np.int64)):
        if a >= 0 and b >= 0 and dyn[a] and dyn[b]:
            ra, rb = find(int(a)), find(int(b))
            if ra != rb:
                parent[max(ra, rb)] = min(ra, rb)
    out = np.full(nb, -1, np.int32)
    ids = {}
    for i in range(nb):
        if dyn[i]:
            r = find(i)
            out[i] = ids.setdefault(r, len(ids))
    return out


def scene_ids(spaces) -> np.ndarray:
    """The scene ids of `spaces` as the int32 array the batched calls take."""
    return np.ascontiguousarray([s.id for s in spaces], dtype=np.int32)


def batch_step(ctx: Context, spaces, dt: float, steps: int = 1, flags: int = N.STEP_ALL):
    """bepugpu_batch_step: every space advances `steps` steps in one batched launch.
    `spaces` is a list of GpuSpace or an int32 array from scene_ids()."""
    ids = spaces if isinstance(spaces, np.ndarray) else scene_ids(spaces)
    ctx.check(ctx.lib.bepugpu_batch_step(ctx.handle, N.ptr(ids), len(ids), float(dt), steps, flags))


def batch_step_each(ctx: Context, spaces, steps, dt: float, flags: int = N.STEP_ALL):
    """bepugpu_batch_step_each: a step count per space."""
    ids = np.ascontiguousarray([s.id for s in spaces], dtype=np.int32)
    k = np.ascontiguousarray(steps, dtype=np.uint32)
    ctx.check(ctx.lib.bepugpu_batch_step_each(ctx.handle, N.ptr(ids), N.ptr(k), len(ids), float(dt), flags))


def set_batch_threads(ctx: Context, threads: int):
    """bepugpu_set_batch_threads: CTA size of batched launches (0 = from the plan)."""
    ctx.check(ctx.lib.bepugpu_set_batch_threads(ctx.handle, int(threads)))


def last_call_stats(ctx: Context):
    """(kernel launches, device ms) of the last batched call."""
    n, ms = ctypes.c_uint32(), ctypes.c_float()
    ctx.check(ctx.lib.bepugpu_last_call_stats(ctx.handle, ctypes.byref(n), ctypes.byref(ms)))
    return n.value, ms.value


def profile_step(space: GpuSpace, dt: float, flags: int = N.STEP_ALL) -> np.ndarray:
    """One instrumented step (bepugpu_profile_step): per-phase device ms and the
    solve census."""
    out = np.zeros(1, N.PHASE_TIMES_DTYPE)
    space.ctx.check(space.ctx.lib.bepugpu_profile_step(space.ctx.handle, space.id, float(dt), flags, N.ptr(out)))
    return out[0]
