"""Batched stepping of many scenes (bepugpu_batch_step) against the oracle and
against stepping each scene on its own."""
import numpy as np
import pytest

import oracle
from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.solver import GpuSpace, batch_step, batch_step_each, default_settings, last_call_stats

from parity import DT, compare

pytestmark = pytest.mark.gpu


def _make(ctx, count=24, seed=9):
    out = []
    sizes = scenes.batch_body_counts(count, 8, 300, seed)
    for i, k in enumerate(sizes):
        b, m, _ = scenes.make_tower(int(k), seed=seed * 1000 + i)
        out.append((b, m, GpuSpace(ctx, b, m)))
    return out


def _oracle_after(b, m, sp, steps):
    o = oracle.OracleSpace(default_settings(), b, m)
    o.set_list_order(sp.colouring()[1])
    o.step(DT, N.STEP_ALL, steps)
    return o.get_bodies(), o.get_constraints()[0]


def test_batch_equals_oracle(gpu_context):
    gpu_context.set_settings(default_settings())
    made = _make(gpu_context)
    batch_step(gpu_context, [sp for _, _, sp in made], DT, steps=3)
    launches, ms = last_call_stats(gpu_context)
    assert launches >= 1 and ms > 0
    for b, m, sp in made:
        ob, om = _oracle_after(b, m, sp, 3)
        gb = sp.download_bodies(b.copy())
        gm, _ = sp.download_constraints(m.copy())
        errs, exact = compare(gb, gm, ob, om)
        assert exact, errs
        sp.close()


def test_batch_each_and_mixed_scenes(gpu_context):
    gpu_context.set_settings(default_settings())
    made = _make(gpu_context, count=10, seed=13)
    # a scene the batched launch cannot take: a free dynamic body outside every island
    b, m, _ = scenes.make_tower(40, seed=77)
    b = np.concatenate([b, b[1:2]])
    b[-1]["position"] = (50.0, 20.0, 50.0)
    free = GpuSpace(gpu_context, b, m)
    made.append((b, m, free))
    steps = [k % 4 for k in range(len(made))]
    batch_step_each(gpu_context, [sp for _, _, sp in made], steps, DT)
    for (b, m, sp), k in zip(made, steps):
        ob, om = _oracle_after(b, m, sp, k)
        gb = sp.download_bodies(b.copy())
        gm, _ = sp.download_constraints(m.copy())
        errs, exact = compare(gb, gm, ob, om)
        assert exact, (k, errs)
        sp.close()


def test_batch_equals_one_scene_steps(gpu_context):
    gpu_context.set_settings(default_settings())
    a = _make(gpu_context, count=6, seed=21)
    c = [(b, m, GpuSpace(gpu_context, b, m)) for b, m, _ in a]
    batch_step(gpu_context, [sp for _, _, sp in a], DT, steps=2)
    for _, _, sp in c:
        sp.step(DT)
        sp.step(DT)
    for (_, _, x), (_, _, y) in zip(a, c):
        np.testing.assert_array_equal(x.download_bodies()["linear_velocity"], y.download_bodies()["linear_velocity"])
        x.close()
        y.close()


def test_batch_errors(gpu_context):
    made = _make(gpu_context, count=2, seed=5)
    sp = made[0][2]
    with pytest.raises(N.ArgumentException):
        batch_step(gpu_context, [sp, sp], DT)
    with pytest.raises(N.ArgumentException):
        batch_step(gpu_context, [sp], 0.0)
    for _, _, s in made:
        s.close()


def test_autotune_keeps_results(gpu_context, tmp_path):
    """Every autotuner setting gives the oracle's bits; the tuned plan is saved and reloaded."""
    from bepuphysics1_gb300 import autotune
    from bepuphysics1_gb300.solver import set_batch_threads
    gpu_context.set_settings(default_settings())
    made = _make(gpu_context, count=12, seed=21)
    spaces = [sp for _, _, sp in made]
    records = [(b, m) for b, m, _ in made]
    res = autotune.tune(gpu_context, spaces, records, DT, targets=(16, 64), budgets=(0, 200 * 1024),
                        threads=(0, 64), steps=(1, 4), calls=1, max_seconds=60)
    assert len(res.trials) >= 5 and res.scene_steps_per_s > 0
    path = tmp_path / "tune.json"
    autotune.save(path, res, "test")
    cfg = autotune.load(path)
    assert cfg == res.best
    for cand in (cfg, autotune.BatchConfig(16, 0, 32, 2)):
        autotune.apply(gpu_context, spaces, records, cand)
        batch_step(gpu_context, spaces, DT, steps=4)
        for b, m, sp in made:
            ob, om = _oracle_after(b, m, sp, 4)
            errs, exact = compare(sp.download_bodies(b.copy()), sp.download_constraints(m.copy())[0], ob, om)
            assert exact, (cand, errs)
    set_batch_threads(gpu_context, 0)
    for sp in spaces:
        sp.close()
