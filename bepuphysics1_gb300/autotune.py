"""Autotuner of the batched path (bepugpu_batch_step).

Four knobs decide how a batch of independent scenes maps onto the GPU:

  target_manifolds  how many manifolds of small islands are packed into one
                    group, i.e. one CTA (bepugpu_set_group_policy);
  smem_budget       the shared-memory residency threshold: a group whose bodies
                    and solve lanes fit it keeps its lanes on chip, larger ones
                    keep them in global memory (bepugpu_set_group_smem_budget);
  threads           CTA size of the batched launches (bepugpu_set_batch_threads);
  steps_per_launch  how many steps one call runs: that many one-step launches
                    captured in one CUDA graph, so the host cost is paid once.

None of them changes results: island groups are independent and each one runs
its manifolds in the list's colour order, so every setting gives the same bits
(the batched tests check this against the oracle and the one-scene path).  The
tuner is coordinate descent over those axes, scored by wall-clock scene-steps/s
of `bepugpu_batch_step` on the caller's own scenes, and its result is a JSON
file that `load` applies later.

The reference has no counterpart: its scene-level parallelism is one Space per
worker (ParallelSpaceTestDemo.cs:24-64).
"""
from __future__ import annotations

import json
import time
from dataclasses import asdict, dataclass, field
from pathlib import Path

from . import native as N
from .solver import Context, GpuSpace, batch_step, last_call_stats, scene_ids, set_batch_threads


@dataclass
class BatchConfig:
    target_manifolds: int = 64
    smem_budget: int = 200 * 1024
    threads: int = 0
    steps_per_launch: int = 1


@dataclass
class Trial:
    config: BatchConfig
    scene_steps_per_s: float
    device_ms_per_launch: float
    launches: int


@dataclass
class TuneResult:
    best: BatchConfig
    scene_steps_per_s: float
    trials: list[Trial] = field(default_factory=list)

    def to_json(self) -> dict:
        return {"best": asdict(self.best), "scene_steps_per_s": self.scene_steps_per_s,
                "trials": [{"config": asdict(t.config), "scene_steps_per_s": t.scene_steps_per_s,
                            "device_ms_per_launch": t.device_ms_per_launch, "launches": t.launches}
                           for t in self.trials]}


TARGETS = (16, 32, 64, 128, 256)
BUDGETS = (0, 48 * 1024, 100 * 1024, 200 * 1024)
THREADS = (0, 32, 64, 128, 256)
STEPS = (1, 2, 4, 8, 16)


def apply_plan(spaces: list[GpuSpace], records, cfg: BatchConfig):
    """Re-plan every scene's island groups for `cfg` and reload its records
    (bodies, manifolds), so that each trial starts from the same state."""
    for sp, (bodies, manifolds) in zip(spaces, records):
        sp.set_group_policy(1, 1024, 4096, cfg.target_manifolds, 0)
        sp.set_group_smem_budget(cfg.smem_budget)
        sp.upload_bodies(bodies)
        sp.upload_constraints(manifolds)


def restore_state(spaces: list[GpuSpace], records):
    """The scenes' bodies and manifolds back to the records, keeping the
    group plan: settling scenes step faster (early-outs), so trials compared
    with one another start from the same state."""
    for sp, (bodies, manifolds) in zip(spaces, records):
        sp.upload_bodies(bodies)
        sp.update_manifolds(manifolds)


def measure(ctx: Context, spaces: list[GpuSpace], dt: float, steps_per_launch: int, calls: int = 3,
            flags: int = N.STEP_ALL) -> Trial:
    """Scene-steps/s of `calls` batched calls after one untimed call (which also
    captures the launch graph)."""
    ids = scene_ids(spaces)
    batch_step(ctx, ids, dt, steps_per_launch, flags)
    dev, t0 = 0.0, time.perf_counter()
    for _ in range(calls):
        batch_step(ctx, ids, dt, steps_per_launch, flags)
        dev += last_call_stats(ctx)[1]
    el = time.perf_counter() - t0
    launches = last_call_stats(ctx)[0]
    return Trial(BatchConfig(), len(spaces) * steps_per_launch * calls / el, dev / calls, launches)


def tune(ctx: Context, spaces: list[GpuSpace], records, dt: float, start: BatchConfig | None = None,
         targets=TARGETS, budgets=BUDGETS, threads=THREADS, steps=STEPS, calls: int = 3,
         max_seconds: float = 60.0) -> TuneResult:
    """Coordinate descent: steps per launch (which amortises the host's cost
    whatever the rest), packing size, residency threshold, then CTA size,
    each axis swept with the others held at their best;
    then packing size and CTA size moved together (twice and half the best
    of both), since the better CTA size follows the packing size.  Every
    trial starts from the records' state.  Stops sweeping once `max_seconds`
    have passed and keeps the best so far."""
    best = BatchConfig(**asdict(start)) if start else BatchConfig()
    trials: list[Trial] = []
    t_begin = time.perf_counter()
    planned = None

    def run(cfg: BatchConfig) -> float:
        nonlocal planned
        key = (cfg.target_manifolds, cfg.smem_budget)
        if planned != key:
            apply_plan(spaces, records, cfg)
            planned = key
        else:
            restore_state(spaces, records)
        set_batch_threads(ctx, cfg.threads)
        t = measure(ctx, spaces, dt, cfg.steps_per_launch, calls)
        t.config = BatchConfig(**asdict(cfg))
        trials.append(t)
        return t.scene_steps_per_s

    best_score = run(best)
    for axis, values in (("steps_per_launch", steps), ("target_manifolds", targets), ("smem_budget", budgets),
                         ("threads", threads)):
        for v in values:
            if getattr(best, axis) == v:
                continue
            if time.perf_counter() - t_begin > max_seconds:
                break
            cand = BatchConfig(**asdict(best))
            setattr(cand, axis, v)
            score = run(cand)
            if score > best_score:
                best, best_score = cand, score
    if best.threads:
        for scale in (2.0, 0.5):
            t, th = int(best.target_manifolds * scale), int(best.threads * scale)
            if t not in targets or th not in threads or time.perf_counter() - t_begin > max_seconds:
                continue
            cand = BatchConfig(**asdict(best))
            cand.target_manifolds, cand.threads = t, th
            score = run(cand)
            if score > best_score:
                best, best_score = cand, score
    # leave the scenes planned for the winner
    if planned != (best.target_manifolds, best.smem_budget):
        apply_plan(spaces, records, best)
    set_batch_threads(ctx, best.threads)
    return TuneResult(best, best_score, trials)


def save(path: str | Path, result: TuneResult, workload: str):
    Path(path).write_text(json.dumps({"workload": workload, **result.to_json()}, indent=1))


def load(path: str | Path) -> BatchConfig:
    return BatchConfig(**json.loads(Path(path).read_text())["best"])


def apply(ctx: Context, spaces: list[GpuSpace], records, cfg: BatchConfig):
    """Use a tuned configuration for these scenes."""
    apply_plan(spaces, records, cfg)
    set_batch_threads(ctx, cfg.threads)
