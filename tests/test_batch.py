"""Batched worlds: one persistent kernel steps many independent worlds.

Every world must evolve exactly as a single world holding the same bodies, so each is
checked bit for bit against its own CPU oracle world.
"""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax


def test_batch_scene_sizes(lib):
    bs = ax.BatchScene(seed=4, worlds=512, median=256, sigma=1.0, min_bodies=16, max_bodies=8192, lib=lib)
    assert bs.sizes.min() >= 16 and bs.sizes.max() <= 8192  # counts include the plane
    assert 180 <= np.median(bs.sizes) <= 360  # lognormal around 256
    assert bs.bodies.n == int(bs.sizes.sum())
    # every world ends with its ground plane
    shapes = bs.bodies.arrays["shape"]
    assert (shapes[bs.offsets[1:] - 1] == ax.SHAPE_PLANE).all()
    again = ax.BatchScene(seed=4, worlds=512, lib=lib)
    assert np.array_equal(again.bodies.arrays["position"], bs.bodies.arrays["position"])


@pytest.mark.gpu
def test_batch_worlds_match_single_world_oracle(gpu_lib, oracle):
    bs = ax.BatchScene(seed=6, worlds=48, median=60, sigma=0.8, min_bodies=16, max_bodies=400, lib=gpu_lib)
    cfg = dict(time_step=1 / 60, velocity_iterations=10)
    batch = ax.Batch(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    batch.set_worlds(bs.bodies, bs.sizes)
    check = sorted({0, 1, int(np.argmax(bs.sizes)), 17, 33, 47})
    worlds = {}
    for w in check:
        o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
        o.add_bodies(bs.world(w))
        worlds[w] = o
    for step in range(25):
        batch.step(1 / 60)
        stats = batch.world_stats()
        for w, o in worlds.items():
            so = o.step(1 / 60)
            assert stats["manifolds"][w] == so.manifold_count, (step, w)
            assert stats["colours"][w] == so.colour_count, (step, w)
    state = batch.read_state()
    for w, o in worlds.items():
        lo, hi = int(bs.offsets[w]), int(bs.offsets[w + 1])
        so = o.read_state()
        for k in state:
            assert np.array_equal(state[k][lo:hi], so[k]), (w, k)
    stats = batch.world_stats()
    assert (stats["flags"] == 0).all()
    assert stats["manifolds"].sum() > 0 and (stats["step_ns"] > 0).all()


@pytest.mark.gpu
def test_batch_tolerance_mode_and_autotune(gpu_lib, oracle, tmp_path):
    bs = ax.BatchScene(seed=9, worlds=24, median=80, sigma=0.5, min_bodies=16, max_bodies=300, lib=gpu_lib)
    cfg = dict(time_step=1 / 60, residual_tolerance=1e-4, max_iterations=400)
    batch = ax.Batch(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    batch.set_worlds(bs.bodies, bs.sizes)
    for _ in range(3):
        batch.step(1 / 60, check=False)
    before = batch.read_state()
    cache = tmp_path / "tune.txt"
    block, ctas = batch.autotune(str(cache), trial_steps=1)
    assert block in (128, 256, 512) and ctas >= 1
    stage = batch.launch()[2]
    assert batch.launch() == (block, ctas, stage) and stage in (0, 1024, 2048, 4096)
    assert cache.read_text().split() == [str(len(bs.sizes)), str(bs.bodies.n), str(block), str(ctas), str(stage)]
    after = batch.read_state()
    for k in before:  # the autotuner restores the state it searched on
        assert np.array_equal(before[k], after[k])
    assert batch.autotune(str(cache)) == (block, ctas)  # cached
    # the tuned batch still matches the oracle world by world
    o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    o.add_bodies(bs.world(5))
    for _ in range(3):
        o.step(1 / 60, check=False)
    for _ in range(4):
        batch.step(1 / 60, check=False)
        so = o.step(1 / 60, check=False)
        st = batch.world_stats()
        assert st["iterations"][5] == so.iterations
    lo, hi = int(bs.offsets[5]), int(bs.offsets[6])
    assert np.array_equal(batch.read_state()["position"][lo:hi], o.read_state()["position"])


@pytest.mark.gpu
def test_batch_big_world_lane_matches_oracle(gpu_lib, oracle):
    # worlds of 4,096 bodies and more run in a concurrent lane of their own (wider CTAs);
    # they must step exactly as single worlds do, and so must the small worlds beside them
    bs = ax.BatchScene(seed=12, worlds=10, median=2500, sigma=0.9, min_bodies=16, max_bodies=8192, lib=gpu_lib)
    sizes = np.asarray(bs.sizes)
    assert (sizes >= 4096).sum() >= 2 and (sizes < 4096).sum() >= 2
    cfg = dict(time_step=1 / 60, velocity_iterations=10)
    batch = ax.Batch(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    batch.set_worlds(bs.bodies, bs.sizes)
    order = np.argsort(sizes)
    check = sorted({int(order[-1]), int(order[-2]), int(order[0])})
    worlds = {}
    for w in check:
        o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
        oracle.oracle_set_threads(o.handle, 8)
        o.add_bodies(bs.world(w))
        worlds[w] = o
    for step in range(8):
        batch.step(1 / 60)
        stats = batch.world_stats()
        for w, o in worlds.items():
            so = o.step(1 / 60)
            assert stats["manifolds"][w] == so.manifold_count, (step, w)
    state = batch.read_state()
    for w, o in worlds.items():
        lo, hi = int(bs.offsets[w]), int(bs.offsets[w + 1])
        so = o.read_state()
        for k in state:
            assert np.array_equal(state[k][lo:hi], so[k]), (w, k)
    assert (batch.world_stats()["flags"] == 0).all()


@pytest.mark.gpu
def test_batch_corrupted_queue_is_reported(gpu_lib):
    """Host-side injected queue faults (a counter that starts late, an entry naming no
    world) make the step return a GPU error instead of silently skipping worlds; the next
    step, with the queue intact again, succeeds.  Nothing faults: the kernel checks each
    entry before use."""
    bs = ax.BatchScene(seed=6, worlds=24, median=60, sigma=0.5, min_bodies=16, max_bodies=300, lib=gpu_lib)
    cfg = dict(time_step=1 / 60, velocity_iterations=4)
    batch = ax.Batch(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    batch.set_worlds(bs.bodies, bs.sizes)
    assert batch.step(1 / 60).status == 0
    for kind, value, code in ((1, 5, ax.ERR_GPU_OPERATION_FAILED), (2, 3, ax.ERR_GPU_INVALID_OPERATION),
                              (1, 0, 0)):
        batch.inject_queue_fault(kind, value)
        st = batch.step(1 / 60, check=False)
        assert st.status == code, (kind, value, st.status)
        assert batch.step(1 / 60).status == 0
    with pytest.raises(ax.AxiomError):
        batch.inject_queue_fault(3, 0)
    with pytest.raises(ax.AxiomError):
        batch.inject_queue_fault(2, 24)


@pytest.mark.gpu
def test_batch_staged_bodies_do_not_change_results(gpu_lib, oracle):
    """Worlds solved with their bodies in shared memory (any staging limit) step exactly as
    with the bodies in global memory, and as the oracle's single worlds."""
    bs = ax.BatchScene(seed=14, worlds=40, median=150, sigma=1.0, min_bodies=16, max_bodies=3000, lib=gpu_lib)
    cfg = dict(time_step=1 / 60, velocity_iterations=10)
    states = []
    for stage in (0, 256, 2048):
        batch = ax.Batch(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
        batch.set_worlds(bs.bodies, bs.sizes)
        batch.set_stage(stage)
        assert batch.launch()[2] == stage
        for _ in range(12):
            batch.step(1 / 60)
        states.append(batch.read_state())
        batch.close()
    for k in states[0]:
        assert np.array_equal(states[0][k], states[1][k]) and np.array_equal(states[0][k], states[2][k]), k
    w = int(np.argmax(bs.sizes))
    o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    oracle.oracle_set_threads(o.handle, 8)
    o.add_bodies(bs.world(w))
    for _ in range(12):
        o.step(1 / 60)
    lo, hi = int(bs.offsets[w]), int(bs.offsets[w + 1])
    so = o.read_state()
    for k in so:
        assert np.array_equal(states[2][k][lo:hi], so[k]), k
    with pytest.raises(ax.AxiomError):
        batch = ax.Batch(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
        batch.set_worlds(bs.bodies, bs.sizes)
        batch.set_stage(5000)
