"""Serving (bepugpu_server_* / bepugpu_serve_*): every result is the same
alone and in the mix, through spills to host memory and back, batched or
plain; the admission and queue limits."""
import threading

import numpy as np
import pytest

from bepuphysics1_gb300 import native as N
from bepuphysics1_gb300 import scenes
from bepuphysics1_gb300.serve import Server
from bepuphysics1_gb300.solver import GpuSpace, default_settings

from parity import DT

pytestmark = pytest.mark.gpu


def _pool(count, seed, lo=16, hi=400):
    sizes = scenes.batch_body_counts(count, lo, hi, seed)
    return [scenes.make_tower(int(k), seed=seed * 1000 + i)[:2] for i, k in enumerate(sizes)]


def _alone(ctx, b, m, steps):
    sp = GpuSpace(ctx, b, m)
    for _ in range(steps):
        sp.step(DT)
    out = sp.download_bodies(b.copy()), sp.download_constraints(m.copy())[0]
    sp.close()
    return out


def _serve(ctx, pool, requests, threads=2, **kw):
    spaces = [GpuSpace(ctx, b, m) for b, m in pool]
    srv = Server(ctx, dt=float(DT), **kw)
    for sp in spaces:
        srv.add(sp)
    done = []
    chunks = [requests[i::threads] for i in range(threads)]

    def submitter(chunk):
        for tag, (i, k) in chunk:
            while srv.submit(spaces[i].id, k, tag) == N.QUEUE_FULL:
                pass

    ts = [threading.Thread(target=submitter, args=(c,)) for c in chunks]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    srv.drain()
    while True:
        c = srv.poll()
        if not len(c):
            break
        done.append(c)
    done = np.concatenate(done) if done else np.zeros(0, N.COMPLETION_DTYPE)
    stats = srv.stats()
    results = []
    for sp, (b, m) in zip(spaces, pool):
        srv.release(sp)
        results.append((sp.download_bodies(b.copy()), sp.download_constraints(m.copy())[0]))
    srv.close()
    for sp in spaces:
        sp.close()
    return results, done, stats


def _requests(n_scenes, n, seed):
    rng = np.random.default_rng(seed)
    return [(t, (int(rng.integers(n_scenes)), int(rng.choice([1, 4, 16])))) for t in range(n)]


def _check_same_alone(ctx, pool, requests, results):
    total = np.zeros(len(pool), int)
    for _, (i, k) in requests:
        total[i] += k
    for i, ((b, m), (gb, gm)) in enumerate(zip(pool, results)):
        ab, am = _alone(ctx, b, m, int(total[i]))
        for f in ("position", "orientation", "linear_velocity", "angular_velocity"):
            np.testing.assert_array_equal(gb[f], ab[f], err_msg=f"scene {i} {f}")
        np.testing.assert_array_equal(gm["contacts"]["penetration_impulse"], am["contacts"]["penetration_impulse"])
        np.testing.assert_array_equal(gm["sliding_impulse"], am["sliding_impulse"])


def test_same_alone_and_in_the_mix(gpu_context):
    gpu_context.set_settings(default_settings())
    pool = _pool(24, 31)
    reqs = _requests(len(pool), 150, 5)
    results, done, stats = _serve(gpu_context, pool, reqs)
    assert len(done) == len(reqs) and np.all(done["status"] == N.OK)
    assert sorted(done["tag"].tolist()) == list(range(len(reqs)))
    assert stats["waves"] >= 1 and stats["spills"] == 0 and stats["pinned_bytes"] == 0
    assert np.all(done["done_us"] >= done["start_us"]) and np.all(done["start_us"] >= done["submit_us"])
    _check_same_alone(gpu_context, pool, reqs, results)


def _resident_bytes(ctx, pool):
    spaces = [GpuSpace(ctx, b, m) for b, m in pool]
    srv = Server(ctx, dt=float(DT))
    for sp in spaces:
        srv.add(sp)
    total = int(srv.stats()["resident_bytes"])
    for sp in spaces:
        srv.release(sp)
        sp.close()
    srv.close()
    return total


def test_spill_and_restore_are_bit_identical(gpu_context):
    gpu_context.set_settings(default_settings())
    pool = _pool(16, 41)
    # a budget that holds about a quarter of the pool forces least-recently-used spills
    budget = _resident_bytes(gpu_context, pool) // 4
    reqs = _requests(len(pool), 120, 7)
    results, done, stats = _serve(gpu_context, pool, reqs, budget_bytes=budget, max_wave_scenes=4)
    assert np.all(done["status"] == N.OK)
    assert stats["spills"] > 0 and stats["restores"] > 0
    # the served set outgrew the budget: spill buffers come from the pinned pool
    assert stats["pinned_bytes"] > 0
    _check_same_alone(gpu_context, pool, reqs, results)


def test_close_with_scenes_spilled(gpu_context):
    """Closing a server restores its spilled scenes before its pinned pool goes:
    the scenes keep their state and step on alone afterwards."""
    gpu_context.set_settings(default_settings())
    pool = _pool(12, 43)
    budget = _resident_bytes(gpu_context, pool) // 3
    spaces = [GpuSpace(gpu_context, b, m) for b, m in pool]
    srv = Server(gpu_context, dt=float(DT), budget_bytes=budget, max_wave_scenes=3)
    for sp in spaces:
        srv.add(sp)
    reqs = _requests(len(pool), 40, 9)
    for tag, (i, k) in reqs:
        while srv.submit(spaces[i].id, k, tag) == N.QUEUE_FULL:
            pass
    srv.drain()
    assert int(srv.stats()["resident_scenes"]) < len(pool)
    srv.close()  # no release: destroy restores every scene
    total = np.zeros(len(pool), int)
    for _, (i, k) in reqs:
        total[i] += k
    for i, (sp, (b, m)) in enumerate(zip(spaces, pool)):
        sp.step(float(DT))  # usable alone again
        gb = sp.download_bodies(b.copy())
        ab, _ = _alone(gpu_context, b, m, int(total[i]) + 1)
        np.testing.assert_array_equal(gb["position"], ab["position"], err_msg=f"scene {i}")
        sp.close()


def test_plain_mode_same_results(gpu_context):
    gpu_context.set_settings(default_settings())
    pool = _pool(10, 51)
    reqs = _requests(len(pool), 60, 9)
    results, done, stats = _serve(gpu_context, pool, reqs, threads=1, batching=False)
    assert np.all(done["status"] == N.OK)
    # one submitter: tags follow submission order, and a scene's requests ran in that order
    by_scene = {}
    for c in np.sort(done, order="tag"):
        by_scene.setdefault(int(c["scene"]), []).append(int(c["wave"]))
    for waves in by_scene.values():
        assert all(a < b for a, b in zip(waves, waves[1:]))
    _check_same_alone(gpu_context, pool, reqs, results)


def test_served_scene_is_locked_and_limits(gpu_context):
    gpu_context.set_settings(default_settings())
    b, m = _pool(1, 61)[0]
    sp = GpuSpace(gpu_context, b, m)
    small = Server(gpu_context, budget_bytes=1024, dt=float(DT))
    with pytest.raises(N.BepuError):  # larger than the budget
        small.add(sp)
    small.close()
    srv = Server(gpu_context, dt=float(DT), queue_capacity=2)
    srv.add(sp)
    with pytest.raises(N.InvalidOperationException):
        sp.step(DT)
    full = accepted = 0
    for t in range(200000):
        st = srv.submit(sp.id, 1, t)
        if st == N.QUEUE_FULL:
            full += 1
            if full > 10:
                break
        else:
            assert st == N.OK
            accepted += 1
    assert full > 0
    got = 0
    while got < accepted:
        got += len(srv.poll())
    srv.drain()
    assert srv.submit(12345678, 1, 0) == N.OK  # unknown scene: completes with NOT_FOUND
    srv.drain()
    c = srv.poll()
    assert len(c) == 1 and c[0]["status"] == N.NOT_FOUND
    srv.release(sp)
    sp.step(DT)
    srv.close()
    sp.close()


def test_context_destroyed_under_a_live_server():
    """Destroying a context stops its servers first (their workers step the
    context's scenes); the server handle then refuses calls but closes."""
    from bepuphysics1_gb300.solver import Context
    ctx = Context(0)
    ctx.set_settings(default_settings())
    pool = _pool(6, 61)
    spaces = [GpuSpace(ctx, b, m) for b, m in pool]
    srv = Server(ctx, dt=float(DT), budget_bytes=_resident_bytes(ctx, pool) // 2, max_wave_scenes=2)
    for sp in spaces:
        srv.add(sp)
    for t, (i, k) in _requests(len(pool), 30, 3):
        while srv.submit(spaces[i].id, k, t) == N.QUEUE_FULL:
            pass
    ctx.close()  # requests may still be queued or running
    with pytest.raises(N.BepuError):
        srv.drain(1000)
    srv.close()


def test_device_heap_reuses_and_returns_memory(gpu_context):
    """Scene arenas are heap blocks: freed blocks are taken again by scenes of
    the same sizes, and slabs no scene uses go back to the device."""
    gpu_context.set_settings(default_settings())
    r0, u0 = gpu_context.memory_usage()
    pool = _pool(40, 71)
    spaces = [GpuSpace(gpu_context, b, m) for b, m in pool]
    r1, u1 = gpu_context.memory_usage()
    assert u1 > u0 and r1 >= u1 and r1 >= r0
    for sp in spaces[::2]:
        sp.close()
    _, u2 = gpu_context.memory_usage()
    assert u0 < u2 < u1
    again = [GpuSpace(gpu_context, b, m) for b, m in pool[::2]]
    r3, u3 = gpu_context.memory_usage()
    assert u3 == u1 and r3 == r1
    for sp in again:
        sp.step(DT)
    for sp in again + spaces[1::2]:
        sp.close()
    assert gpu_context.memory_usage() == (r0, u0)


def test_served_scenes_spill_into_held_heap(gpu_context):
    """While a server lives its spills keep the heap's slabs; they go back when
    the server and the scenes are gone."""
    gpu_context.set_settings(default_settings())
    r0, u0 = gpu_context.memory_usage()
    pool = _pool(12, 72)
    spaces = [GpuSpace(gpu_context, b, m) for b, m in pool]
    _, u1 = gpu_context.memory_usage()
    srv = Server(gpu_context, budget_bytes=(u1 - u0) // 3, dt=float(DT))
    for sp in spaces:
        srv.add(sp)
    for k in range(3):
        for sp in spaces:
            while srv.submit(sp.id, 1, k) == N.QUEUE_FULL:
                srv.poll()
    srv.drain()
    st = srv.stats()
    assert st["spills"] > 0 and st["restores"] > 0
    r2, u2 = gpu_context.memory_usage()
    assert u2 < u1 and r2 >= r0
    srv.close()
    for sp in spaces:
        sp.close()
    assert gpu_context.memory_usage() == (r0, u0)
