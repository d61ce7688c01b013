#!/usr/bin/env python
"""Benchmark of the GB300 solver step on the 65,536-box pile.

One step = ContactRefresher -> ForceUpdater -> Solver (prestep, warm start,
10 iterations) -> PositionUpdater over the pile's frozen manifold set
(65,536 manifolds, 262,144 contacts), float32.  The metric is contact-iters/s
= sum over manifolds of contacts x iterations, per second.

  value       device time of K steps (CUDA events on the scene stream around
              each graph launch), inputs resident in HBM, L2 flushed between
              steps by writing a 512 MiB buffer (the step's working set is
              below L2 size).
  e2e         the same metric through the C ABI with host buffers
              (bepugpu_step_state): every step sends every body's state from
              pinned host memory, steps, and brings back every body's state and
              every manifold's contact ids and impulses; host wall clock.  The
              whole-record path (bepugpu_step_host) and the separate calls are
              reported beside it.
  roofline    the dominant kernel: k_groups when island groups run the step
              (algorithmic bytes of the units one launch processes: executed
              solve visits counted by a census, warm start, prestep, bodies),
              else k_solve (76 d + 136 + 48 c per executed manifold visit);
              divided by the kernel's device time from events captured in the
              step graph; peak = measured HBM copy bandwidth.  `sweep` adds
              the colour-sweep path's k_solve on the same pile, groups off.
  cpu_baseline the oracle port of Solver.UpdateMultithreaded (per-body spin
              locks, chunked parallel loop) on all host cores, on a bounded
              sample of steps of the same pile.
  dropped     the same pile dropped from a 2 m grid and settled for 120 steps
              with the device broad phase, narrow phase and solver, then its
              captured manifold set timed like the headline.
  islands     device ms of a step of the pile's 4,096 column islands awake and
              asleep (DeactivationManager on the device).

`--impl reference` times that CPU port alone (the reference is C# and no .NET
runtime exists on these machines).  Under torchrun every rank steps its own
replica of the pile ("replicas only": a single scene does not shard); rank 0
prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

DT = np.float32(1 / 60)
WORKLOAD = "pile_64k"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--mode", default="graph", choices=["graph", "persistent"])
    ap.add_argument("--persistent-blocks", type=int, default=1)
    ap.add_argument("--groups", default="on", choices=["on", "off"],
                    help="island groups: whole steps of small islands in one CTA")
    ap.add_argument("--group-target", type=int, default=64, help="manifolds packed per group CTA")
    ap.add_argument("--group-threads", type=int, default=0, help="threads per group CTA (0 = from the plan)")
    ap.add_argument("--group-prologue", type=int, default=-1, choices=[-1, 0, 1],
                    help="island groups' refresh, body updates and prestep: 0 in the group kernel, "
                         "1 as grid-wide launches before it, -1 by scene size")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-seconds", type=float, default=10.0)
    ap.add_argument("--no-batch", action="store_true", help="skip the many-scene batching section")
    ap.add_argument("--batch-scenes", type=int, default=4096)
    ap.add_argument("--batch-rounds", type=int, default=5, help="timed rounds of the plain and batched paths")
    ap.add_argument("--tune-seconds", type=float, default=30.0, help="autotuner time limit")
    ap.add_argument("--tune-out", default=None, help="write the autotuner's trials to this JSON file")
    ap.add_argument("--batch-cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-chains", action="store_true", help="skip the mixed joints-and-contacts section")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving section")
    ap.add_argument("--no-collide", action="store_true", help="skip the narrow-phase section")
    ap.add_argument("--no-sweep", action="store_true", help="skip the colour-sweep path section")
    ap.add_argument("--no-pile1k", action="store_true", help="skip the 1,000-box pile section")
    ap.add_argument("--no-dropped", action="store_true", help="skip the dropped-and-settled pile section")
    ap.add_argument("--dropped-steps", type=int, default=240, help="settling steps of the dropped pile")
    ap.add_argument("--no-islands", action="store_true", help="skip the simulation-islands section")
    ap.add_argument("--pile1k-cpu-seconds", type=float, default=2.0)
    ap.add_argument("--collide-cpu-seconds", type=float, default=8.0)
    ap.add_argument("--serve-scenes", type=int, default=16384)
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="arrival window per load level")
    ap.add_argument("--serve-waves", type=int, default=4, help="batched waves in flight (1..4)")
    ap.add_argument("--serve-wave-scenes", type=int, default=4096, help="scenes per batched wave at most")
    ap.add_argument("--serve-rates", default="1000,20000,100000,200000",
                    help="Poisson arrival rates (requests/s)")
    ap.add_argument("--serve-plain-rates", default="1000,20000")
    ap.add_argument("--serve-spill-rates", default="1000,20000",
                    help="arrival rates under a device budget of half the served bytes")
    ap.add_argument("--chain-cpu-seconds", type=float, default=8.0)
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def measured_hbm_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def ncu_traffic_per_launch(kernel: str, workload: str = "pile64k"):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/<kernel>_<workload>.md), if any."""
    p = ROOT / "profiles" / f"{kernel}_{workload}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def step_static_bytes(bodies, manifolds):
    """Algorithmic bytes of a step beside the solve visits (the per-step
    formula's warm-start, prestep and body terms): per manifold with a contact
    and a dynamic body, one warm-start visit 76 d + 136 + 48 c and a prestep
    64 d + 136 + 56 c; 152 per dynamic body (force and position updates)."""
    dyn = np.asarray(bodies["is_dynamic"]) != 0
    a, b = np.asarray(manifolds["body_a"]), np.asarray(manifolds["body_b"])
    da = (a >= 0) & dyn[np.clip(a, 0, None)]
    db = (b >= 0) & dyn[np.clip(b, 0, None)]
    d = da.astype(np.int64) + db.astype(np.int64)
    c = np.asarray(manifolds["contact_count"]).astype(np.int64)
    live = (d > 0) & (c > 0)
    warm = float((76 * d + 136 + 48 * c)[live].sum())
    prestep = float((64 * d + 136 + 56 * c)[live].sum())
    return warm, prestep, 152.0 * float(dyn.sum())


def cpu_baseline(bodies, manifolds, contact_iters_per_step, seconds, threads):
    """The oracle's port of Solver.UpdateMultithreaded on `threads` host cores."""
    import oracle
    from bepuphysics1_gb300 import native as N
    from bepuphysics1_gb300.solver import default_settings
    o = oracle.OracleSpace(default_settings(), bodies, manifolds)
    o.set_order_mode(oracle.ORDER_PERMUTED, 0)
    o.step_multithreaded(DT, N.STEP_ALL, 1, threads)  # warm-up step (MultithreadedScalingTestDemo.cs:223)
    steps, t0 = 0, time.perf_counter()
    while True:
        o.step_multithreaded(DT, N.STEP_ALL, 1, threads)
        steps += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    o.close()
    return {"value": contact_iters_per_step * steps / dt, "unit": "contact-iters/s", "cores": threads,
            "kind": "port", "steps": steps,
            "sample": f"{steps} full steps of the 65,536-box pile after 1 warm-up step "
                      f"(oracle port of Solver.UpdateMultithreaded, {threads} threads, {dt:.1f} s)"}


def timed_steps(space, steps, flush, flags):
    """Device ms of `steps` steps (events in the step graph) and of their
    solve phase, with L2 flushed before each."""
    import torch
    from bepuphysics1_gb300 import native as N
    step_ms, solve_ms = [], []
    for _ in range(steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        space.step(DT, flags)
        step_ms.append(space.last_step_ms())
        solve_ms.append(float(space.last_step_phase_ms()[3]))
    torch.cuda.synchronize()
    return step_ms, solve_ms


def solve_roofline(prof, solve_ms, peak, peak_kind):
    """k_solve: the executed manifold visits' algorithmic bytes (census) over
    the solve phase's device time, one launch per colour sweep."""
    bytes_per_step = float(prof["solve_algorithmic_bytes"])
    launches = int(prof["solve_launches"])
    mean_s = statistics.mean(solve_ms) / 1000.0
    achieved = bytes_per_step / mean_s / 1e9 if mean_s > 0 else 0.0
    return {"bound": "hbm", "kernel": "k_solve", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": bytes_per_step / max(launches, 1),
            "algorithmic": "76 d + 136 + 48 c per executed manifold visit",
            "launch_ms_avg": 1000.0 * mean_s / max(launches, 1), "solve_launches_per_step": launches,
            "solve_ms_per_step": 1000.0 * mean_s,
            "manifold_visits_per_step": float(prof["solve_manifold_visits"])}


def sweep_section(args, ctx, local, pg, peak, peak_kind):
    """The colour-sweep path (one launch per colour, one thread per manifold):
    the 65,536-box pile with island groups off, and the pile packed as config
    1 packs its 1,000 boxes (unit boxes at 1.05 m, +-0.05 m jitter) scaled to
    64 x 16 x 64, whose touching columns make one island too large for a
    group, so the default policy sweeps it."""
    import torch
    from bepuphysics1_gb300 import native as N
    from bepuphysics1_gb300 import scenes
    from bepuphysics1_gb300.solver import GpuSpace, profile_step
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    out = {}
    cases = [("pile_64k_groups_off", scenes.pile_64k, (0, 1024, 4096, 64, 0)),
             ("pile_64k_packed", lambda: scenes.make_pile(nx=64, ny=16, nz=64, spacing=1.05, size_min=1.0,
                                                         size_max=1.0, jitter=0.05, friction_min=0.6,
                                                         friction_max=0.6, seed=11), None)]
    for name, make, policy in cases:
        bodies, manifolds, _ = make()
        space = GpuSpace(ctx, bodies, manifolds, group_policy=policy) if policy else GpuSpace(ctx, bodies, manifolds)
        for _ in range(max(args.warmup, 3)):
            space.step(DT, N.STEP_ALL)
        ctx.synchronize()
        live_m, _ = space.download_constraints()
        cips = int(live_m["contact_count"].sum()) * int(ctx.settings["iteration_limit"])
        if pg:
            pg.barrier()
        step_ms, solve_ms = timed_steps(space, args.steps, flush, N.STEP_ALL)
        prof = profile_step(space, DT, N.STEP_ALL)
        ms = statistics.mean(step_ms)
        out[name] = {"value": cips / (ms / 1000.0), "unit": "contact-iters/s", "ms_per_step": ms,
                     "bodies": int(len(bodies)), "manifolds": int(len(manifolds)),
                     "contacts": int(live_m["contact_count"].sum()), "colours": int(space.colouring()[2]),
                     "group_ctas": int(prof["groups"]), "gpu_launches_per_step": int(space.last_step_launches()),
                     "roofline": solve_roofline(prof, solve_ms, peak, peak_kind)}
        space.close()
    out["l2"] = "flushed between timed steps (512 MiB write)"
    return out


def dropped_section(args, ctx, local, pg):
    """Config 2 as written: pile_64k's 65,536 boxes on a 64 x 16 x 64 grid
    with 2 m between layers too, dropped onto the ground and settled with the
    device broad phase and pair bookkeeping (bepugpu_update_pairs: records
    and colouring on the device), the device narrow phase and the solver.  120 steps (2 s) are not enough for
    the top layers, which fall about 16 m, to land: the state after 120 steps
    is reported and the pile settles for --dropped-steps in all.  Then the
    settled heap's pair set, its contacts regenerated by the narrow phase each
    step, timed like the headline (contact-iters/s, I = 10)."""
    import torch
    from bepuphysics1_gb300 import native as N
    from bepuphysics1_gb300 import scenes
    from bepuphysics1_gb300.solver import GpuSpace, islands_of
    bodies, shapes, friction = scenes.dropped_pile()
    nb = len(bodies)
    space = GpuSpace(ctx, bodies, None, capacity=(nb, 8 * nb, 0), shapes=shapes)
    space.set_materials(np.stack([friction, friction, np.zeros_like(friction)], 1))
    flags = N.STEP_ALL | N.STEP_COLLIDE
    loop_ms, counts, after120 = [], [], None
    t0 = time.perf_counter()
    for step in range(args.dropped_steps):
        if step == 120:
            b120 = space.download_bodies(bodies.copy())
            d120 = b120["is_dynamic"] == 1
            sp120 = np.linalg.norm(b120["linear_velocity"][d120], axis=1)
            after120 = {"speed_p50": float(np.median(sp120)), "speed_p99": float(np.percentile(sp120, 99)),
                        "top": float(b120["position"][d120][:, 1].max())}
        ts = time.perf_counter()
        counts.append(space.update_pairs(DT))  # pair bookkeeping and recolouring on the device
        space.step(DT, flags)
        ctx.synchronize()
        loop_ms.append(1000.0 * (time.perf_counter() - ts))
    settle_s = time.perf_counter() - t0
    gb = space.download_bodies(bodies.copy())
    gm, _ = space.download_constraints()
    space.close()
    dyn = gb["is_dynamic"] == 1
    speed = np.linalg.norm(gb["linear_velocity"][dyn], axis=1)
    # the settled heap's pair set kept, its contacts regenerated every step by the narrow phase
    isl = islands_of(gb, gm)
    sizes = np.bincount(isl[isl >= 0]) if (isl >= 0).any() else np.zeros(1, np.int64)
    solved = GpuSpace(ctx, gb, gm, shapes=shapes)
    for _ in range(max(args.warmup, 3)):
        solved.step(DT, flags)
    ctx.synchronize()
    live_m, _ = solved.download_constraints()
    contacts = int(live_m["contact_count"].sum())
    cips = contacts * int(ctx.settings["iteration_limit"])
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    if pg:
        pg.barrier()
    step_ms, _ = timed_steps(solved, args.steps, flush, flags)
    from bepuphysics1_gb300.solver import profile_step
    prof = profile_step(solved, DT, flags)
    ms = statistics.mean(step_ms)
    launches = int(solved.last_step_launches())
    # the same steps in the persistent cooperative kernel (grid barriers between sweeps)
    solved.set_mode(N.MODE_PERSISTENT)
    for _ in range(3):
        solved.step(DT, flags)
    pers_ms, _ = timed_steps(solved, args.steps, flush, flags)
    solved.set_mode(N.MODE_GRAPH)
    out = {"workload": "pile_64k dropped from a 64 x 16 x 64 grid (2 m spacing) and settled for "
                       f"{args.dropped_steps} steps on the device",
           "value": cips / (ms / 1000.0), "unit": "contact-iters/s", "ms_per_step": ms,
           "step": "collide+refresh+forces+solve+positions on the settled heap's pair set",
           "bodies": int(nb), "manifolds": int(len(gm)), "contacts": contacts,
           "colours": int(solved.colouring()[2]), "islands": int(isl.max() + 1) if (isl >= 0).any() else 0,
           "largest_island": int(sizes.max()), "group_ctas": int(prof["groups"]),
           "gpu_launches_per_step": launches, "persistent_ms_per_step": statistics.mean(pers_ms),
           "settle": {"steps": args.dropped_steps, "seconds": settle_s, "manifolds_final": counts[-1],
                      "loop_ms_median": statistics.median(loop_ms),
                      "loop_ms_last20_median": statistics.median(loop_ms[-20:]),
                      "after_120_steps": after120,
                      "what": "per step: bepugpu_update_pairs (device broad phase, pair records and "
                              "recolouring on the device), then the narrow phase + solver step; host wall clock",
                      "speed_p50_after": float(np.median(speed)), "speed_p99_after": float(np.percentile(speed, 99)),
                      "top_after": float(gb["position"][dyn][:, 1].max())},
           "parity": "the same loop bit-exact against the oracle on a 5 x 4 x 5 drop (tests/test_gpu_settle.py)",
           "l2": "flushed between timed steps (512 MiB write)"}
    solved.close()
    return out


def islands_section(args, ctx, local, pg):
    """Simulation islands on the device: 4,096 columns of 16 unit cubes as
    islands (IsAlwaysActive cleared), stepped until every island sleeps (the
    round robin looks at 100 members' worth of islands a step); device ms of
    a step with every island awake and with every island asleep."""
    import torch
    from bepuphysics1_gb300 import native as N
    from bepuphysics1_gb300 import scenes
    from bepuphysics1_gb300.solver import GpuSpace, islands_of
    # unit cubes, so that every column stands (pile_64k's random sizes topple
    # some columns, which never come to rest on a frozen manifold set)
    bodies, manifolds, _ = scenes.make_pile(nx=64, ny=16, nz=64, spacing=2.0, size_min=1.0, size_max=1.0,
                                            jitter=0.02, friction_min=0.6, friction_max=0.6,
                                            ground_size=(140.0, 1.0, 140.0), seed=5)
    bodies = bodies.copy()
    bodies["activity"] &= ~np.uint32(N.BODY_ALWAYS_ACTIVE)
    space = GpuSpace(ctx, bodies, manifolds)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    for _ in range(3):
        space.step(DT, N.STEP_ALL)
    plain_ms, _ = timed_steps(space, args.steps, flush, N.STEP_ALL)  # no islands: every island awake
    space.upload_bodies(bodies)
    isl = islands_of(bodies, manifolds)
    space.set_islands(isl)
    awake_ms, _ = timed_steps(space, args.steps, flush, N.STEP_ALL)
    steps = args.steps
    asleep_at = None
    for k in range(4000):
        space.step(DT, N.STEP_ALL)
        steps += 1
        if k % 50 == 49:
            f, _ = space.get_islands()
            if not np.any(f & N.ISLAND_ACTIVE):
                asleep_at = steps
                break
    if pg:
        pg.barrier()
    asleep_ms, _ = timed_steps(space, args.steps, flush, N.STEP_ALL)
    f, idx = space.get_islands()
    launches = int(space.last_step_launches())
    space.close()
    batched = islands_batch(args, ctx)
    out = {"workload": "64 x 16 x 64 unit cubes in 4,096 column islands", "islands": int(len(f)),
           "without_islands_ms_per_step": statistics.mean(plain_ms),
           "awake_ms_per_step": statistics.mean(awake_ms), "asleep_ms_per_step": statistics.mean(asleep_ms),
           "all_asleep_after_steps": asleep_at, "asleep_now": int(np.count_nonzero((f & N.ISLAND_ACTIVE) == 0)),
           "launches_per_step": launches,
           "what": "DeactivationManager.Update on the device (1 launch without moving kinematic bodies, 2 with) "
                   "before the group step; a group whose "
                   "islands all sleep returns after loading its bodies",
           "l2": "flushed between timed steps (512 MiB write)", "batched_columns": batched}
    return out


def islands_batch(args, ctx):
    """1,024 scenes of four columns of eight unit cubes with islands through
    bepugpu_batch_step, 8 steps a call: scene-steps/s while awake and once
    their islands sleep (a group whose islands all sleep returns at once)."""
    from bepuphysics1_gb300 import native as N
    from bepuphysics1_gb300 import scenes
    from bepuphysics1_gb300.solver import GpuSpace, batch_step, islands_of, last_call_stats
    spaces = []
    for i in range(1024):
        b, m, _ = scenes.make_pile(nx=2, ny=8, nz=2, spacing=2.0, size_min=1.0, size_max=1.0, jitter=0.02,
                                   friction_min=0.6, friction_max=0.6, ground_size=(10.0, 1.0, 10.0), seed=12000 + i)
        b = b.copy()
        b["activity"] &= ~np.uint32(N.BODY_ALWAYS_ACTIVE)
        sp = GpuSpace(ctx, b, m)
        sp.set_islands(islands_of(b, m))
        spaces.append(sp)
    steps = 8

    def timed(calls):
        ms = []
        for _ in range(calls):
            batch_step(ctx, spaces, DT, steps)
            ms.append(last_call_stats(ctx)[1])
        return statistics.median(ms)

    for _ in range(3):
        batch_step(ctx, spaces, DT, steps)
    awake_ms = timed(5)
    calls, asleep_share = 8, 0.0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < 20.0:
        batch_step(ctx, spaces, DT, steps)
        calls += 1
        if calls % 25 == 0:
            flags = np.concatenate([sp.get_islands()[0] for sp in spaces])
            asleep_share = float(np.mean((flags & N.ISLAND_ACTIVE) == 0))
            if asleep_share > 0.99:
                break
    asleep_ms = timed(5)
    flags = np.concatenate([sp.get_islands()[0] for sp in spaces])
    for sp in spaces:
        sp.close()
    n = len(spaces)
    return {"scenes": n, "steps_per_call": steps, "awake_scene_steps_per_s": n * steps / (awake_ms / 1000.0),
            "asleep_scene_steps_per_s": n * steps / (asleep_ms / 1000.0), "awake_ms_per_call": awake_ms,
            "asleep_ms_per_call": asleep_ms, "islands_asleep": float(np.mean((flags & N.ISLAND_ACTIVE) == 0)),
            "steps_until_measured": calls * steps}


def pile1k_section(args, ctx, local, pg):
    """The 1,000-box pile (unit boxes at 1.05 m, +-0.05 m jitter, I = 10): the
    one-scene GPU step beside the oracle port's single-threaded
    (Solver.UpdateSingleThreaded, PermutationMapper order) and multithreaded
    (Solver.UpdateMultithreaded, all host cores) steps, each CPU leg a bounded
    sample of whole steps."""
    import torch
    import oracle
    from bepuphysics1_gb300 import native as N
    from bepuphysics1_gb300 import scenes
    from bepuphysics1_gb300.solver import GpuSpace, default_settings
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    bodies, manifolds, _ = scenes.pile_1k()
    space = GpuSpace(ctx, bodies, manifolds)
    for _ in range(max(args.warmup, 3)):
        space.step(DT, N.STEP_ALL)
    ctx.synchronize()
    live_m, _ = space.download_constraints()
    cips = int(live_m["contact_count"].sum()) * int(ctx.settings["iteration_limit"])
    if pg:
        pg.barrier()
    step_ms, _ = timed_steps(space, args.steps, flush, N.STEP_ALL)
    ms = statistics.mean(step_ms)
    space.close()
    out = {"workload": "pile_1k", "bodies": int(len(bodies)), "manifolds": int(len(manifolds)),
           "contacts": int(live_m["contact_count"].sum()),
           "gpu": {"value": cips / (ms / 1000.0), "unit": "contact-iters/s", "ms_per_step": ms,
                   "path": "bepugpu_step, one scene, island groups (device time, L2 flushed)"}}
    if args.no_cpu_baseline:
        return out
    threads = os.cpu_count() or 1
    for name, nthreads in (("cpu_single_thread", 1), ("cpu_multithreaded", threads)):
        o = oracle.OracleSpace(default_settings(), bodies, manifolds)
        o.set_order_mode(oracle.ORDER_PERMUTED, 0)

        def one_step():
            if nthreads > 1:
                o.step_multithreaded(DT, N.STEP_ALL, 1, nthreads)
            else:
                o.step(DT, N.STEP_ALL, 1)

        one_step()  # warm-up step (MultithreadedScalingTestDemo.cs:223)
        steps, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < args.pile1k_cpu_seconds:
            one_step()
            steps += 1
        el = time.perf_counter() - t0
        o.close()
        out[name] = {"value": cips * steps / el, "unit": "contact-iters/s", "cores": nthreads, "kind": "port",
                     "ms_per_step": 1000 * el / steps,
                     "sample": f"{steps} steps after 1 warm-up step (oracle port of Solver.Update"
                               f"{'Multithreaded' if nthreads > 1 else 'SingleThreaded'}, {el:.1f} s)"}
    return out


BATCH_WORKLOAD = "towers_4096"
BATCH_ITERATIONS = 8


def batch_records(n, rank=0, world=1):
    """The many-scene workload: n tower scenes, body counts log-uniform in
    [8, 2048]; a rank takes every world-th scene."""
    from bepuphysics1_gb300 import scenes
    sizes = scenes.batch_body_counts(n, 8, 2048, 4)
    return [scenes.make_tower(int(k), seed=4 * 100003 + i)[:2] for i, k in enumerate(sizes) if i % world == rank]


def batch_settings():
    from bepuphysics1_gb300.solver import default_settings
    s = default_settings()
    s["iteration_limit"] = BATCH_ITERATIONS
    return s


def cpu_batch_baseline(records, seconds, threads):
    """Scene-parallel CPU stepping (ParallelSpaceTestDemo.cs:64): one oracle
    Space per scene, single-threaded each, scenes spread over `threads` host
    threads; one untimed round, then whole rounds until `seconds` pass."""
    from concurrent.futures import ThreadPoolExecutor
    import oracle
    from bepuphysics1_gb300 import native as N
    settings = batch_settings()
    spaces = [oracle.OracleSpace(settings, b, m) for b, m in records]
    for o in spaces:
        o.set_order_mode(oracle.ORDER_PERMUTED, 0)

    def one(o):
        o.step(DT, N.STEP_ALL, 1)

    rounds = 0
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(one, spaces))
        t0 = time.perf_counter()
        while True:
            list(ex.map(one, spaces))
            rounds += 1
            if time.perf_counter() - t0 >= seconds:
                break
        el = time.perf_counter() - t0
    for o in spaces:
        o.close()
    return {"value": len(records) * rounds / el, "unit": "scene-steps/s", "cores": threads, "kind": "port",
            "sample": f"{rounds} rounds of all {len(records)} scenes after 1 warm-up round, one single-threaded "
                      f"oracle Space per scene on {threads} threads ({el:.1f} s)"}


def batch_section(args, local, rank, world, pg):
    """Config-4 workload: the plain one-scene-per-launch path (bepugpu_step on
    every scene) against batched stepping (bepugpu_batch_step) at the
    autotuned configuration.  Both are timed on the host clock around calls
    that return with the work finished; results are bit-identical between the
    two paths (tests/test_gpu_batch.py)."""
    from bepuphysics1_gb300 import autotune
    from bepuphysics1_gb300 import native as N
    from bepuphysics1_gb300.solver import Context, GpuSpace

    t0 = time.perf_counter()
    records = batch_records(args.batch_scenes, rank, world)
    ctx = Context(local, batch_settings())
    spaces = [GpuSpace(ctx, b, m) for b, m in records]
    setup_s = time.perf_counter() - t0
    n = len(spaces)
    bodies = sum(len(b) for b, _ in records)
    manifolds = sum(len(m) for _, m in records)
    contacts = sum(int(m["contact_count"].sum()) for _, m in records)

    def barrier():
        if pg:
            pg.barrier()

    # autotuned batched path (every trial starts from the records' state)
    # the search starts from the best setting of earlier tunings of this mix
    res = autotune.tune(ctx, spaces, records, DT, start=autotune.BatchConfig(128, 100 * 1024, 128, 16),
                        max_seconds=args.tune_seconds)
    if args.tune_out:
        autotune.save(args.tune_out, res, BATCH_WORKLOAD)
    best = res.best
    K = best.steps_per_launch
    calls = max(args.batch_rounds, 3)

    def from_records():
        """The records' state, then 3 warm-up steps on the plain path: the
        plain and the batched timings start from the same scene state."""
        autotune.restore_state(spaces, records)
        for _ in range(3):
            for sp in spaces:
                sp.step(DT, N.STEP_ALL)
        ctx.synchronize()

    # plain path: one bepugpu_step per scene, each its own graph launch, over
    # the same steps as the batched timing (after K untimed steps, the batched
    # path's graph-capturing first call)
    from_records()
    for _ in range(K):
        for sp in spaces:
            sp.step(DT, N.STEP_ALL)
    ctx.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(calls * K):
        for sp in spaces:
            sp.step(DT, N.STEP_ALL)
    ctx.synchronize()
    plain_s = time.perf_counter() - t0
    plain_steps = calls * K
    plain_launches = sum(sp.last_step_launches() for sp in spaces)

    per_k = {}
    for k in sorted({1, K}):
        from_records()
        barrier()
        per_k[k] = autotune.measure(ctx, spaces, DT, k, calls=calls)
    tb = per_k[K]
    t1 = per_k[1]

    def whole(v):
        if not pg:
            return v
        import torch
        x = torch.tensor([v], dtype=torch.float64, device=f"cuda:{local}")
        pg.all_reduce(x)
        return float(x.item())

    plain_rate = whole(n * plain_steps / plain_s)
    batched_rate = whole(tb.scene_steps_per_s)
    batched_1 = whole(t1.scene_steps_per_s)

    # roofline of the batched launches: the step formula's algorithmic bytes of
    # every scene (solve visits from a census of one instrumented step each)
    # per scene-step, times the scene-steps of a call, over its device time
    from bepuphysics1_gb300.solver import profile_step
    step_bytes = 0.0
    for sp, (b, _) in zip(spaces, records):
        prof = profile_step(sp, DT, N.STEP_ALL)
        live_m, _ = sp.download_constraints()
        warm_b, prestep_b, body_b = step_static_bytes(b, live_m)
        step_bytes += float(prof["solve_algorithmic_bytes"]) + float(prof["group_solve_algorithmic_bytes"]) + \
            warm_b + prestep_b + body_b
    peak, peak_kind = measured_hbm_peak()
    call_bytes = step_bytes * best.steps_per_launch
    achieved = call_bytes / (tb.device_ms_per_launch / 1000.0) / 1e9 if tb.device_ms_per_launch > 0 else 0.0
    # ncu's DRAM bytes of one launch over the first 512 scenes of the mix, scaled
    # by manifolds to this launch's scenes (each scene's records move about once)
    traffic = ncu_traffic_per_launch("k_batch_groups", "towers512")
    if traffic is not None:
        first512 = records[:512] if world == 1 and n >= 512 else batch_records(512)
        traffic = traffic * manifolds / max(sum(len(m) for _, m in first512), 1)
    batch_roofline = {"bound": "hbm", "kernel": "k_batch_groups", "achieved": achieved, "peak": peak,
                      "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                      "traffic": None if traffic is None else traffic * K,
                      "traffic_note": "ncu DRAM bytes of one launch over 512 scenes (profiles/"
                                      "k_batch_groups_towers512.md) scaled by manifolds to this call's scenes, "
                                      "times its launches",
                      "algorithmic_bytes_per_call": call_bytes, "device_ms_per_call": tb.device_ms_per_launch,
                      "launches_per_call": tb.launches,
                      "algorithmic": "per scene-step: 76 d + 136 + 48 c per executed solve visit (census), one "
                                     "warm-start visit and one prestep per active manifold, 152 per dynamic body"}
    out = {
        "metric": "scene-steps/s", "workload": BATCH_WORKLOAD,
        "config": {"scenes": args.batch_scenes, "bodies": bodies, "manifolds": manifolds, "contacts": contacts,
                   "body_counts": "log-uniform in [8, 2048], towers of height 4..32 on a per-scene ground",
                   "iterations": BATCH_ITERATIONS, "dt": float(DT), "setup_s": setup_s},
        "plain": {"value": plain_rate, "unit": "scene-steps/s", "rounds": plain_steps,
                  "ms_per_round": 1000 * plain_s / plain_steps, "gpu_launches_per_round": int(plain_launches),
                  "path": "bepugpu_step per scene (one graph launch per scene-step), host clock"},
        "window": f"both paths from the records' state: 3 warm-up steps, {K} untimed steps, then the "
                  f"{calls * K} timed steps ({calls} batched calls of {K}); the 1-step-per-launch figure "
                  f"times steps 5..{4 + calls}",
        "batched": {"value": batched_rate, "unit": "scene-steps/s", "steps_per_launch": best.steps_per_launch,
                    "ms_per_call": 1000 * n * best.steps_per_launch / tb.scene_steps_per_s,
                    "device_ms_per_call": tb.device_ms_per_launch, "gpu_launches_per_call": tb.launches,
                    "path": "bepugpu_batch_step, host clock around calls that return finished"},
        "batched_1_step_per_launch": {"value": batched_1, "unit": "scene-steps/s",
                                      "device_ms_per_call": t1.device_ms_per_launch,
                                      "gpu_launches_per_call": t1.launches},
        "roofline": batch_roofline,
        "speedup_vs_plain": batched_rate / plain_rate,
        "speedup_vs_plain_1_step_per_launch": batched_1 / plain_rate,
        "contact_iters_per_s_batched": contacts * BATCH_ITERATIONS * batched_rate / max(args.batch_scenes, 1),
        "autotune": {"best": autotune.asdict(best), "trials": len(res.trials),
                     "table": [[t.config.target_manifolds, t.config.smem_budget, t.config.threads,
                                t.config.steps_per_launch, round(t.scene_steps_per_s)] for t in res.trials],
                     "columns": ["target_manifolds", "smem_budget", "threads", "steps_per_launch",
                                 "scene_steps_per_s"]},
        "equal_error": "bit-identical to the plain path and to the colour-ordered oracle",
    }
    for sp in spaces:
        sp.close()
    ctx.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_batch_baseline(records, args.batch_cpu_seconds, os.cpu_count() or 1)
    return out


CHAIN_WORKLOAD = "chains_8k"
CHAIN_ITERATIONS = 15


def chain_section(args, local, rank, world, pg):
    """Mixed joints and contacts: 8,192 chains of 16 capsules joined alternately
    by BallSocketJoint + SwingLimit and RevoluteJoint (limit active, +-45
    degrees), plus 20,000 loose spheres and boxes, 15 iterations.  Device time
    per step with L2 flushed between steps; the unit of work is one solver
    visit of one updateable (joint or manifold) per iteration."""
    import torch
    from bepuphysics1_gb300 import native as N
    from bepuphysics1_gb300 import scenes
    from bepuphysics1_gb300.solver import Context, GpuSpace, default_settings
    settings = default_settings()
    settings["iteration_limit"] = CHAIN_ITERATIONS
    bodies, manifolds, joints = scenes.chains_8k()
    ctx = Context(local, settings)
    sp = GpuSpace(ctx, bodies, manifolds, joints)
    for _ in range(max(args.warmup, 3)):
        sp.step(DT, N.STEP_ALL)
    ctx.synchronize()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    step_ms, solve_ms = [], []
    if pg:
        pg.barrier()
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        sp.step(DT, N.STEP_ALL)
        step_ms.append(sp.last_step_ms())
        solve_ms.append(float(sp.last_step_phase_ms()[3]))
    total_ms = float(sum(step_ms))
    if pg:
        t = torch.tensor([total_ms], device=f"cuda:{local}")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        total_ms = float(t.item())
    n_upd = len(joints) + len(manifolds)
    contacts = scenes.contact_count(manifolds)
    colours = sp.colouring()[2]
    out = {
        "metric": "updateable-iters/s", "workload": CHAIN_WORKLOAD,
        "value": world * n_upd * CHAIN_ITERATIONS * args.steps / (total_ms / 1000.0), "unit": "updateable-iters/s",
        "steps_per_s": world * args.steps / (total_ms / 1000.0), "ms_per_step": total_ms / args.steps,
        "solve_ms_per_step": statistics.mean(solve_ms), "gpu_launches_per_step": int(sp.last_step_launches()),
        "config": {"bodies": int(len(bodies)), "joints": int(len(joints)), "manifolds": int(len(manifolds)),
                   "contacts": int(contacts), "iterations": CHAIN_ITERATIONS, "colours": int(colours),
                   "joint_records": {name: int((joints["type"] == t).sum()) for name, t in
                                     (("ball_socket", N.JOINT_BALL_SOCKET), ("swing_limit", N.JOINT_SWING_LIMIT),
                                      ("revolute", N.JOINT_REVOLUTE))},
                   "l2": "flushed between timed steps (512 MiB write)"},
        "parity": "bit-exact vs the colour-ordered oracle (tests/test_gpu_joints.py)",
    }
    # roofline of the step (its launches are the joint-island group kernels):
    # manifold visits from a census, joint visits counted as joints x
    # iterations (an upper bound: joints that early-out are counted), each
    # 76 d + 256 bytes (its 13 solve lanes and state read, 2 impulse lanes and
    # state written, each moving body's velocities and inertia); warm start,
    # prestep and body terms as the step formula has them
    from bepuphysics1_gb300.solver import profile_step
    prof = profile_step(sp, DT, N.STEP_ALL)
    live_m, _ = sp.download_constraints()
    warm_b, prestep_b, body_b = step_static_bytes(bodies, live_m)
    dyn = np.asarray(bodies["is_dynamic"]) != 0
    ja, jb = np.asarray(joints["body_a"]), np.asarray(joints["body_b"])
    jd = ((ja >= 0) & dyn[np.clip(ja, 0, None)]).astype(np.int64) + ((jb >= 0) & dyn[np.clip(jb, 0, None)])
    joint_visit_bytes = float((76 * jd + 256).sum())
    step_bytes = float(prof["solve_algorithmic_bytes"]) + float(prof["group_solve_algorithmic_bytes"]) + \
        warm_b + prestep_b + body_b + joint_visit_bytes * (CHAIN_ITERATIONS + 2)  # + warm start and prestep
    peak, peak_kind = measured_hbm_peak()
    achieved = step_bytes / (total_ms / args.steps / 1000.0) / 1e9
    # bepugpu_set_group_prologue's default: groups holding joints and >= 8,192 constraints are split
    out["split_prologue"] = len(joints) + len(manifolds) >= 8192
    out["roofline"] = {"bound": "hbm", "kernel": "k_groups (joint islands)" + (
                           ", after k_group_refresh_force and k_group_prestep" if out["split_prologue"] else ""),
                       "achieved": achieved, "peak": peak,
                       "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                       "algorithmic_bytes_per_step": step_bytes,
                       "algorithmic": "manifolds: the step formula with a census of solve visits; joints: "
                                      "76 d + 256 per visit, joints x (iterations + 2) visits (upper bound)"}
    sp.close()

    # the same scene with its joints re-typed as ten of the added joint, limit and motor types
    mixed = scenes.with_added_joint_types(bodies, joints)
    sp = GpuSpace(ctx, bodies, manifolds, mixed)
    for _ in range(max(args.warmup, 3)):
        sp.step(DT, N.STEP_ALL)
    ctx.synchronize()
    mixed_ms = []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        sp.step(DT, N.STEP_ALL)
        mixed_ms.append(sp.last_step_ms())
    mixed_total = float(sum(mixed_ms))
    if pg:
        t = torch.tensor([mixed_total], device=f"cuda:{local}")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        mixed_total = float(t.item())
    out["added_types"] = {
        "value": world * n_upd * CHAIN_ITERATIONS * args.steps / (mixed_total / 1000.0), "unit": "updateable-iters/s",
        "steps_per_s": world * args.steps / (mixed_total / 1000.0), "ms_per_step": mixed_total / args.steps,
        "gpu_launches_per_step": int(sp.last_step_launches()),
        "joint_types": sorted({int(t) for t in mixed["type"]}),
        "what": "chains_8k with its joints re-typed in turn as weld, distance, prismatic with its limit, revolute "
                "motor, linear servo motor, maximum speed, twist limit, swivel hinge, ellipse swing limit and "
                "point on plane (scenes.with_added_joint_types)",
    }
    sp.close()
    ctx.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        threads = os.cpu_count() or 1
        o = oracle.OracleSpace(settings, bodies, manifolds, mixed)
        o.set_order_mode(oracle.ORDER_PERMUTED, 0)
        o.step_multithreaded(DT, N.STEP_ALL, 1, threads)
        steps, t0 = 0, time.perf_counter()
        while True:
            o.step_multithreaded(DT, N.STEP_ALL, 1, threads)
            steps += 1
            if time.perf_counter() - t0 >= args.chain_cpu_seconds / 2:
                break
        el = time.perf_counter() - t0
        o.close()
        out["added_types"]["cpu_baseline"] = {"steps_per_s": steps / el, "cores": threads, "kind": "port",
                                              "sample": f"{steps} steps of the oracle port, {threads} threads"}
        o = oracle.OracleSpace(settings, bodies, manifolds, joints)
        o.set_order_mode(oracle.ORDER_PERMUTED, 0)
        o.step_multithreaded(DT, N.STEP_ALL, 1, threads)
        steps, t0 = 0, time.perf_counter()
        while True:
            o.step_multithreaded(DT, N.STEP_ALL, 1, threads)
            steps += 1
            if time.perf_counter() - t0 >= args.chain_cpu_seconds:
                break
        el = time.perf_counter() - t0
        o.close()
        out["cpu_baseline"] = {"value": n_upd * CHAIN_ITERATIONS * steps / el, "unit": "updateable-iters/s",
                               "steps_per_s": steps / el, "cores": threads, "kind": "port",
                               "sample": f"{steps} full steps after 1 warm-up step (oracle port of "
                                         f"Solver.UpdateMultithreaded, {threads} threads, {el:.1f} s)"}
    return out


COLLIDE_WORKLOAD = "pile_64k_collide"


def collide_section(args, local, rank, world, pg):
    """The full step with the narrow phase on the device: the 65,536-box pile
    with every pair an empty GENERATED manifold, so each step regenerates the
    contacts from the poses (BoxBoxCollider + BoxContactManifold id matching)
    before the solver.  Device time per step with L2 flushed between steps;
    the narrow phase alone is timed as steps of the collide stage only."""
    import torch
    from bepuphysics1_gb300 import native as N
    from bepuphysics1_gb300 import scenes
    from bepuphysics1_gb300.solver import Context, GpuSpace, default_settings
    settings = default_settings()
    bodies, manifolds, _, shapes = scenes.pile_64k_collide()
    ctx = Context(local, settings)
    sp = GpuSpace(ctx, bodies, manifolds, shapes=shapes)
    for _ in range(max(args.warmup, 3)):
        sp.step(DT, N.STEP_ALL)
    ctx.synchronize()
    gm, _ = sp.download_constraints()
    contacts = int(gm["contact_count"].sum())
    iters = int(settings["iteration_limit"])
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    step_ms, collide_ms = [], []
    if pg:
        pg.barrier()
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        sp.step(DT, N.STEP_ALL)
        step_ms.append(sp.last_step_ms())
    launches = int(sp.last_step_launches())
    for _ in range(args.steps):  # the narrow phase alone over the same poses
        flush.fill_(1)
        torch.cuda.synchronize()
        sp.step(DT, N.STEP_COLLIDE)
        collide_ms.append(sp.last_step_ms())
    total_ms = float(sum(step_ms))
    if pg:
        t = torch.tensor([total_ms], device=f"cuda:{local}")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        total_ms = float(t.item())
    pairs = len(manifolds)
    cms = statistics.mean(collide_ms)
    # algorithmic bytes of one pair: head, two shapes, two poses, impulses and
    # the kept contacts' four lanes read (144 + 64 c), the same lanes of the new
    # contacts and the impulses written (32 + 64 c); c = 4 on the resting pile
    c_avg = contacts / max(pairs, 1)
    pair_bytes = 176 + 128 * c_avg
    peak, peak_kind = measured_hbm_peak()
    achieved = pairs * pair_bytes / (cms / 1000.0) / 1e9
    out = {
        "metric": "contact-iters/s", "workload": COLLIDE_WORKLOAD,
        "value": world * contacts * iters * args.steps / (total_ms / 1000.0), "unit": "contact-iters/s",
        "ms_per_step": total_ms / args.steps, "steps_per_s": world * args.steps / (total_ms / 1000.0),
        "narrow_phase": {"pairs_per_s": world * pairs / (cms / 1000.0), "ms_per_launch": cms,
                         "kernel": "k_collide", "share_of_step": cms / (total_ms / args.steps),
                         "roofline": {"bound": "latency (per-pair SAT and clipping in registers and local "
                                               "memory)", "algorithmic_bytes_per_pair": pair_bytes,
                                      "achieved": achieved, "peak": peak, "unit": "GB/s",
                                      "frac": achieved / peak, "peak_kind": peak_kind}},
        "gpu_launches_per_step": launches,
        "config": {"bodies": int(len(bodies)), "pairs": pairs, "contacts_after_warmup": contacts,
                   "iterations": iters, "step": "collide+refresh+forces+solve+positions",
                   "l2": "flushed between timed steps (512 MiB write)"},
        "parity": "bit-exact vs the oracle's narrow phase and solver (tests/test_gpu_collide.py)",
    }
    # the broad phase over the same bodies: the overlapping pairs, sorted
    sp.broad_phase(DT)  # first call sizes its buffers
    bp_ms = []
    for _ in range(max(3, min(args.steps, 10))):
        t0 = time.perf_counter()
        bp_pairs = sp.broad_phase(DT)
        bp_ms.append(1000 * (time.perf_counter() - t0))
    out["broad_phase"] = {"ms_per_call": statistics.median(bp_ms), "pairs": int(len(bp_pairs)),
                          "bodies_per_s": len(bodies) / (statistics.median(bp_ms) / 1000.0),
                          "path": "bepugpu_broad_phase: boxes, uniform-grid cell entries sorted on the device, "
                                  "pairs within cells, pairs sorted on the device and copied back; host clock "
                                  "per call",
                          "parity": "the oracle's brute-force pair set (tests/test_gpu_broad_phase.py)"}
    sp.close()
    ctx.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        threads = os.cpu_count() or 1
        o = oracle.OracleSpace(settings, bodies, manifolds, shapes=shapes)
        o.set_order_mode(oracle.ORDER_PERMUTED, 0)
        o.step_multithreaded(DT, N.STEP_ALL, 1, threads)
        steps, t0 = 0, time.perf_counter()
        while True:
            o.step_multithreaded(DT, N.STEP_ALL, 1, threads)
            steps += 1
            if time.perf_counter() - t0 >= args.collide_cpu_seconds:
                break
        el = time.perf_counter() - t0
        o.close()
        out["cpu_baseline"] = {"value": contacts * iters * steps / el, "unit": "contact-iters/s",
                               "steps_per_s": steps / el, "cores": threads, "kind": "port",
                               "sample": f"{steps} full steps with the narrow phase after 1 warm-up step "
                                         f"(oracle port, {threads} threads, {el:.1f} s)"}
    return out


SERVE_WORKLOAD = "serve_16k"
SERVE_ITERATIONS = 8
SERVE_GROUP_MANIFOLDS = 128  # the batch autotuner's best for the tower mix
SERVE_THREADS = 128


def serve_records(n, rank=0, world=1):
    """The serving pool: n tower scenes, body counts log-uniform in [16, 4096]."""
    from bepuphysics1_gb300 import scenes
    sizes = scenes.batch_body_counts(n, 16, 4096, 5)
    return [scenes.make_tower(int(k), seed=5 * 100003 + i)[:2] for i, k in enumerate(sizes) if i % world == rank]


def poisson_load(srv, ids, rate, seconds, seed):
    """Submits Poisson arrivals at `rate` requests/s for `seconds` (each a uniform
    choice of scene and of k in {1, 4, 16} steps) while a second thread polls
    completions; returns the completions and the achieved submit rate."""
    import threading
    from bepuphysics1_gb300 import native as N
    rng = np.random.default_rng(seed)
    n = max(1, int(rate * seconds))
    gaps = rng.exponential(1.0 / rate, n)
    when = np.cumsum(gaps)
    scene = rng.integers(0, len(ids), n)
    steps = rng.choice(np.array([1, 4, 16]), n)
    out, stop = [], threading.Event()

    def poller():
        while not stop.is_set():
            c = srv.poll()
            if len(c):
                out.append(c)
            else:
                time.sleep(0.0005)

    th = threading.Thread(target=poller)
    th.start()
    t0 = time.perf_counter()
    full = 0
    for i in range(n):
        while time.perf_counter() - t0 < when[i]:
            pass
        while srv.submit(ids[scene[i]], int(steps[i]), i) == N.QUEUE_FULL:
            full += 1
    submit_s = time.perf_counter() - t0
    srv.drain(600000)
    stop.set()
    th.join()
    while True:
        c = srv.poll()
        if not len(c):
            break
        out.append(c)
    done = np.concatenate(out) if out else np.zeros(0, N.COMPLETION_DTYPE)
    return done, n / submit_s, full


def serve_level(srv, ids, rate, seconds, seed):
    from bepuphysics1_gb300 import native as N
    s0 = srv.stats()
    done, achieved, full = poisson_load(srv, ids, rate, seconds, seed)
    s1 = srv.stats()
    ok = done[done["status"] == N.OK]
    lat = (ok["done_us"] - ok["submit_us"]) / 1000.0
    span_s = (ok["done_us"].max() - ok["submit_us"].min()) / 1e6 if len(ok) else 1.0
    waves = int(s1["waves"] - s0["waves"])
    return {"rate": rate, "achieved_rate": achieved, "requests": int(len(done)), "ok": int(len(ok)),
            "scene_steps_per_s": float(ok["steps"].sum()) / span_s,
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "max_ms": float(lat.max()) if len(lat) else None,
            "queue_ms_p50": float(np.percentile((ok["start_us"] - ok["submit_us"]) / 1000.0, 50)) if len(ok) else None,
            "waves": waves, "scenes_per_wave": float(s1["wave_scenes"] - s0["wave_scenes"]) / max(waves, 1),
            "launches": int(s1["launches"] - s0["launches"]), "spills": int(s1["spills"] - s0["spills"]),
            "restores": int(s1["restores"] - s0["restores"]), "submit_ring_full": int(full),
            "spill_ms": (int(s1["spill_us"]) - int(s0["spill_us"])) / 1e3,
            "restore_ms": (int(s1["restore_us"]) - int(s0["restore_us"])) / 1e3,
            "room_waits": int(s1["room_waits"] - s0["room_waits"]),
            "failed": int(len(done) - len(ok)), "last_error": srv.last_error() if len(done) > len(ok) else None}


def serve_section(args, local, rank, world, pg):
    """Serving workload: a pool of tower scenes resident on the device, Poisson
    step requests (k in {1, 4, 16}) at swept arrival rates, p50/p99 request
    latency (submit to completion seen, host steady clock) and sustained
    scene-steps/s; continuously batched against plain one-launch-per-step
    serving, and once under a device budget of half the pool (LRU spills)."""
    from bepuphysics1_gb300.serve import Server
    from bepuphysics1_gb300.solver import Context, GpuSpace

    t0 = time.perf_counter()
    records = serve_records(args.serve_scenes, rank, world)
    settings = batch_settings()
    settings["iteration_limit"] = SERVE_ITERATIONS
    ctx = Context(local, settings)
    # the batch autotuner's setting for towers (128 manifolds per group, 128-thread
    # batched CTAs); the plain path steps the same group plans with their own CTA sizes
    spaces = [GpuSpace(ctx, b, m, group_policy=(1, 1024, 4096, SERVE_GROUP_MANIFOLDS, 0)) for b, m in records]
    setup_s = time.perf_counter() - t0
    ids = [sp.id for sp in spaces]
    rates = [float(r) for r in args.serve_rates.split(",") if r]
    plain_rates = [float(r) for r in args.serve_plain_rates.split(",") if r]
    out = {"metric": "scene-steps/s and request latency", "workload": SERVE_WORKLOAD,
           "config": {"scenes": args.serve_scenes, "bodies": int(sum(len(b) for b, _ in records)),
                      "manifolds": int(sum(len(m) for _, m in records)),
                      "body_counts": "log-uniform in [16, 4096], towers of height 4..32",
                      "iterations": SERVE_ITERATIONS, "k": [1, 4, 16], "arrival_window_s": args.serve_seconds,
                      "group_manifolds": SERVE_GROUP_MANIFOLDS, "batched_threads": SERVE_THREADS,
                      "batched_waves_in_flight": args.serve_waves, "batched_wave_scenes": args.serve_wave_scenes,
                      "setup_s": setup_s, "latency": "submit to completion seen by the server, steady clock"}}

    def run(mode_rates, **kw):
        t_run = time.perf_counter()
        srv = Server(ctx, dt=float(DT), **kw)
        t_add = time.perf_counter()
        for sp in spaces:
            srv.add(sp)
        t_add = time.perf_counter() - t_add
        # warm-up: one 1-step request per scene (first launches, one-scene graphs), untimed
        for i in ids:
            while srv.submit(i, 1, 0) != 0:
                srv.poll()
        srv.drain(600000)
        while len(srv.poll()):
            pass
        t_warm = time.perf_counter() - t_add - t_run
        st = srv.stats()
        warm = {"s": t_warm, "waves": int(st["waves"]), "spills": int(st["spills"]), "restores": int(st["restores"]),
                "spill_ms": int(st["spill_us"]) / 1e3, "restore_ms": int(st["restore_us"]) / 1e3}
        if rank == 0:
            print(f"bench: serve {kw} warm-up {warm}", file=sys.stderr, flush=True)
        levels = [serve_level(srv, ids, r, args.serve_seconds, 17 + i) for i, r in enumerate(mode_rates)]
        res = {"levels": levels, "resident_bytes": int(st["resident_bytes"]),
               "resident_scenes": int(st["resident_scenes"]), "pinned_spill_bytes": int(st["pinned_bytes"]),
               "add_scenes_s": t_add, "warmup": warm, "run_s": time.perf_counter() - t_run}
        srv.close()
        return res

    out["batched"] = run(rates, batching=True, budget_bytes=120 << 30, threads=SERVE_THREADS,
                         waves_in_flight=args.serve_waves, max_wave_scenes=args.serve_wave_scenes)
    out["batched"]["device_budget_bytes"] = 120 << 30
    out["plain"] = run(plain_rates, batching=False, budget_bytes=120 << 30)
    total = out["batched"]["resident_bytes"]
    spill_rate = [float(r) for r in args.serve_spill_rates.split(",") if r]
    out["batched_half_budget"] = run(spill_rate, batching=True, budget_bytes=max(total // 2, 1 << 20),
                                     threads=SERVE_THREADS)
    out["batched_half_budget"]["device_budget_bytes"] = max(total // 2, 1 << 20)
    by_rate = {lv["rate"]: lv for lv in out["plain"]["levels"]}
    out["vs_plain"] = [{"rate": lv["rate"], "p99_ms_batched": lv["p99_ms"],
                        "p99_ms_plain": by_rate[lv["rate"]]["p99_ms"],
                        "scene_steps_per_s_batched": lv["scene_steps_per_s"],
                        "scene_steps_per_s_plain": by_rate[lv["rate"]]["scene_steps_per_s"]}
                       for lv in out["batched"]["levels"] if lv["rate"] in by_rate]
    out["equal_error"] = "bit-identical to stepping each scene alone (tests/test_gpu_serve.py)"
    for sp in spaces:
        sp.close()
    ctx.close()
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from bepuphysics1_gb300 import scenes
    from bepuphysics1_gb300.solver import default_settings
    import oracle
    from bepuphysics1_gb300 import native as N
    threads = os.cpu_count() or 1
    bodies, manifolds, _ = scenes.pile_64k()
    iters = int(default_settings()["iteration_limit"])
    cips = scenes.contact_count(manifolds) * iters
    o = oracle.OracleSpace(default_settings(), bodies, manifolds)
    o.set_order_mode(oracle.ORDER_PERMUTED, 0)
    for _ in range(max(args.warmup, 1)):
        o.step_multithreaded(DT, N.STEP_ALL, 1, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step_multithreaded(DT, N.STEP_ALL, 1, threads)
    el = time.perf_counter() - t0
    value = cips * args.steps / el
    line = {
        "metric": "contact-iters/s", "value": value, "unit": "contact-iters/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "bodies": int(len(bodies)), "manifolds": int(len(manifolds)),
                   "contacts": int(scenes.contact_count(manifolds)), "iterations": iters, "dt": float(DT),
                   "order": "PermutationMapper (Solver.cs:255-260)"},
        "cpu_baseline": {"value": value, "unit": "contact-iters/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full steps of the pile after {max(args.warmup, 1)} warm-up steps; "
                                   "C++ port of Solver.UpdateMultithreaded (the C# reference has no runtime here)"},
        "e2e": {"value": value, "unit": "contact-iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import __graft_entry__
    t_start = time.perf_counter()
    section_s = {}

    def mark(name, since):
        section_s[name] = round(time.perf_counter() - since, 2)
        if rank == 0:
            print(f"bench: {name} {section_s[name]:.1f} s", file=sys.stderr, flush=True)
        return time.perf_counter()

    __graft_entry__.build()
    from bepuphysics1_gb300 import native as N
    from bepuphysics1_gb300 import scenes
    from bepuphysics1_gb300.solver import Context, GpuSpace, default_settings, profile_step

    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist

    t_sec = mark("build", t_start)
    bodies, manifolds, _ = scenes.pile_64k()
    settings = default_settings()
    iters = int(settings["iteration_limit"])
    ctx = Context(local, settings)
    policy = (0 if args.groups == "off" else 1, 1024, 4096, args.group_target, args.group_threads)
    space = GpuSpace(ctx, bodies, manifolds, group_policy=policy)
    space.set_group_prologue(args.group_prologue)
    space.set_mode(N.MODE_GRAPH if args.mode == "graph" else N.MODE_PERSISTENT)
    if args.mode == "persistent":
        ctx.check(ctx.lib.bepugpu_set_persistent_blocks_per_sm(ctx.handle, space.id, args.persistent_blocks))
    colours = space.colouring()[2]
    # bepugpu_set_group_prologue(-1) splits only groups holding joints: the pile's stay in the kernel
    split_prologue = args.groups == "on" and args.group_prologue == 1

    for _ in range(max(args.warmup, 3)):
        space.step(DT, N.STEP_ALL)
    ctx.synchronize()
    live_m, _ = space.download_constraints()
    contacts = int(live_m["contact_count"].sum())
    cips = contacts * iters  # contact-iterations per step

    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    step_ms, solve_ms, group_ms = [], [], []
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            space.step(DT, N.STEP_ALL)
            step_ms.append(space.last_step_ms())
            phases = space.last_step_phase_ms()
            solve_ms.append(float(phases[3]))
            group_ms.append(float(phases[5]))
    torch.cuda.synchronize()
    total_ms = float(sum(step_ms))
    launches = space.last_step_launches() * args.steps
    if pg:
        t = torch.tensor([total_ms], device=f"cuda:{local}")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        total_ms = float(t.item())
        pg.barrier()
    value = world * cips * args.steps / (total_ms / 1000.0)

    # roofline of the dominant kernel, from a census of one instrumented step
    prof = profile_step(space, DT, N.STEP_ALL)
    peak, peak_kind = measured_hbm_peak()
    kernel_only = {k: float(prof[k]) for k in ("refresh_ms", "force_ms", "prestep_ms", "warm_ms", "solve_ms",
                                               "position_ms", "group_ms")}
    warm_b, prestep_b, body_b = step_static_bytes(bodies, live_m)
    step_alg = float(prof["solve_algorithmic_bytes"]) + warm_b + prestep_b + body_b
    step_achieved = step_alg / (total_ms / args.steps / 1000.0) / 1e9
    if int(prof["groups"]) > 0 and statistics.mean(group_ms) >= statistics.mean(solve_ms):
        # Island groups: one launch runs whole steps of the small islands.  Its
        # algorithmic bytes are the step formula over the units it processes:
        # its executed solve visits (census), one warm-start visit and one
        # prestep per active manifold, force and position per body.  With the
        # sweep part empty (every manifold in a group) all of the step is its.
        group_visits = float(prof["group_solve_algorithmic_bytes"])
        share = 1.0 if int(prof["solve_launches"]) == 0 else \
            float(prof["group_solve_manifold_visits"]) / max(float(prof["solve_manifold_visits"]), 1.0)
        bytes_per_launch = group_visits + share * (warm_b + prestep_b + body_b)
        launch_s = statistics.mean(group_ms) / 1000.0
        achieved = bytes_per_launch / launch_s / 1e9
        floor = float(prof["group_compulsory_bytes"])
        roofline = {"bound": "hbm", "kernel": "k_groups", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_kind": peak_kind, "traffic": ncu_traffic_per_launch("k_groups"),
                    "algorithmic_bytes_per_launch": bytes_per_launch,
                    "algorithmic": "76 d + 136 + 48 c per executed solve visit and per warm-start visit, "
                                   "64 d + 136 + 56 c per prestep, 152 per dynamic body",
                    "launch_ms_avg": 1000.0 * launch_s, "launches_per_step": 1, "ctas": int(prof["groups"]),
                    "manifold_visits_per_step": float(prof["group_solve_manifold_visits"]),
                    "dram_floor_bytes_per_launch": floor,
                    "dram_floor_frac": floor / launch_s / 1e9 / peak,
                    "dram_floor": "each input lane read once and each output lane written once "
                                  "(136 + 64 c per manifold with shared-memory lanes, 208 per body)",
                    "kernel_only_ms_per_step": kernel_only}
    else:
        bytes_per_step = float(prof["solve_algorithmic_bytes"])
        solve_launches = int(prof["solve_launches"])
        mean_solve_s = statistics.mean(solve_ms) / 1000.0 if solve_ms else float(prof["solve_ms"]) / 1000.0
        achieved = bytes_per_step / mean_solve_s / 1e9 if mean_solve_s > 0 else 0.0
        roofline = {"bound": "hbm", "kernel": "k_solve", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_kind": peak_kind, "traffic": ncu_traffic_per_launch("k_solve"),
                    "algorithmic_bytes_per_launch": bytes_per_step / max(solve_launches, 1),
                    "algorithmic": "76 d + 136 + 48 c per executed manifold visit",
                    "launch_ms_avg": 1000.0 * mean_solve_s / max(solve_launches, 1),
                    "solve_launches_per_step": solve_launches,
                    "manifold_visits_per_step": float(prof["solve_manifold_visits"]),
                    "kernel_only_ms_per_step": kernel_only}
    roofline["step"] = {"algorithmic_bytes_per_step": step_alg, "achieved": step_achieved,
                        "frac": step_achieved / peak, "ms_per_step": total_ms / args.steps,
                        "what": "the whole step (every kernel, launch gaps included) against the same bytes"}

    t_sec = mark("headline", t_sec)
    # e2e through the C ABI with pinned host records
    e2e = None
    if not args.no_e2e:
        hb = torch.empty(bodies.nbytes, dtype=torch.uint8, pin_memory=True).numpy().view(N.BODY_DTYPE)
        hm = torch.empty(manifolds.nbytes, dtype=torch.uint8, pin_memory=True).numpy().view(N.MANIFOLD_DTYPE)
        # downloads fill the state fields of existing records: start from the scene's records
        hb[:] = bodies
        hm[:] = manifolds
        space.download_bodies(hb)
        space.download_constraints(hm)
        ctx.synchronize()
        k = max(3, min(args.steps, 10))
        # state records: the bodies' state up, one step, the bodies' state and
        # the manifolds' impulses down (bepugpu_step_state)
        sb = torch.empty(len(bodies) * N.BODY_STATE_DTYPE.itemsize, dtype=torch.uint8,
                         pin_memory=True).numpy().view(N.BODY_STATE_DTYPE)
        sm = torch.empty(len(manifolds) * N.MANIFOLD_STATE_DTYPE.itemsize, dtype=torch.uint8,
                         pin_memory=True).numpy().view(N.MANIFOLD_STATE_DTYPE)
        space.download_state(sb, sm)
        space.step_state(sb, sm, DT, N.STEP_ALL)  # untimed: first call of the path
        if pg:
            pg.barrier()
        t2 = time.perf_counter()
        for _ in range(k):
            space.step_state(sb, sm, DT, N.STEP_ALL)
        el_state = time.perf_counter() - t2
        space.download_bodies(hb)
        space.download_constraints(hm)
        if pg:
            pg.barrier()
        t0 = time.perf_counter()
        for _ in range(k):
            space.step_host(hb, hm, DT, N.STEP_ALL)
        el = time.perf_counter() - t0
        # the same through the separate calls (update, step, download), for comparison
        t1 = time.perf_counter()
        for _ in range(k):
            space.update_bodies(hb)
            space.update_manifolds(hm)
            space.step(DT, N.STEP_ALL)
            space.download_bodies(hb)
            space.download_constraints(hm)
        el_calls = time.perf_counter() - t1
        h2d = hb.nbytes + hm.nbytes
        d2h = hb.nbytes + hm.nbytes  # whole body and manifold records come back
        e2e = {"value": world * cips * k / el_state, "unit": "contact-iters/s",
               "h2d_bytes_per_step": int(sb.nbytes), "d2h_bytes_per_step": int(sb.nbytes + sm.nbytes),
               "steps": k, "ms_per_step": 1000 * el_state / k,
               "path": "bepugpu_step_state (every body's state up from pinned host memory, one step, every "
                       "body's state and every manifold's contact ids and impulses down; host wall clock)",
               "whole_records": {"value": world * cips * k / el, "ms_per_step": 1000 * el / k,
                                 "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                                 "path": "bepugpu_step_host (body and manifold records up, checked, one step, "
                                         "whole records down)"},
               "separate_calls": {"value": world * cips * k / el_calls, "ms_per_step": 1000 * el_calls / k,
                                  "path": "update_bodies, update_manifolds, step, download_bodies, "
                                          "download_constraints"}}

    t_sec = mark("e2e", t_sec)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(bodies, manifolds, cips, args.cpu_sample_seconds, os.cpu_count() or 1)
    t_sec = mark("cpu_baseline", t_sec)

    sweep = None
    if not args.no_sweep:
        space.close()
        sweep = sweep_section(args, ctx, local, pg, peak, peak_kind)
        off = sweep["pile_64k_groups_off"]
        roofline["sweep"] = {"kernel": "k_solve", "workload": "pile_64k, island groups off",
                             "frac": off["roofline"]["frac"], "achieved": off["roofline"]["achieved"],
                             "ms_per_step": off["ms_per_step"],
                             "solve_ms_per_step": off["roofline"]["solve_ms_per_step"],
                             "packed_pile_frac": sweep["pile_64k_packed"]["roofline"]["frac"]}
        t_sec = mark("sweep", t_sec)
    pile1k = None
    if not args.no_pile1k:
        space.close()
        pile1k = pile1k_section(args, ctx, local, pg)
        t_sec = mark("pile1k", t_sec)
    dropped = None
    if not args.no_dropped:
        space.close()
        dropped = dropped_section(args, ctx, local, pg)
        t_sec = mark("dropped", t_sec)
    islands = None
    if not args.no_islands:
        space.close()
        islands = islands_section(args, ctx, local, pg)
        t_sec = mark("islands", t_sec)
    batch = None
    if not args.no_batch:
        space.close()
        batch = batch_section(args, local, rank, world, pg)
        t_sec = mark("batch", t_sec)
    chains = None
    if not args.no_chains:
        space.close()
        chains = chain_section(args, local, rank, world, pg)
        t_sec = mark("chains", t_sec)
    collide = None
    if not args.no_collide:
        space.close()
        collide = collide_section(args, local, rank, world, pg)
        t_sec = mark("collide", t_sec)
    serve = None
    if not args.no_serve:
        space.close()
        serve = serve_section(args, local, rank, world, pg)
        t_sec = mark("serve", t_sec)
    section_s["total"] = round(time.perf_counter() - t_start, 2)

    if rank == 0:
        line = {
            "metric": "contact-iters/s", "value": value, "unit": "contact-iters/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "bodies": int(len(bodies)), "manifolds": int(len(manifolds)),
                       "contacts": contacts, "iterations": iters, "colours": int(colours), "dt": float(DT),
                       "step": "refresh+forces+solve+positions", "mode": args.mode,
                       "island_groups": {"enabled": args.groups == "on", "ctas": int(prof["groups"]),
                                         "target_manifolds": args.group_target,
                                         "threads": args.group_threads or "plan",
                                         "prologue": "grid-wide launches" if split_prologue
                                         else "in the group kernel"},
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "flushed between timed steps (512 MiB write)"},
            "gpu_launches": int(launches),
            "roofline": roofline,
            "sweep": sweep,
            "pile_1k": pile1k,
            "dropped": dropped,
            "islands": islands,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "batch": batch,
            "chains": chains,
            "collide": collide,
            "serve": serve,
            "section_seconds": section_s,
        }
        print(json.dumps(line), flush=True)
    space.close()
    ctx.close()
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
