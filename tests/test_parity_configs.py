"""GPU vs CPU oracle at the configured workload sizes, not scaled-down ones.

  C3  the 1,048,576-sphere walled pile (the benchmark's workload: temporally coherent
      colouring, linear slop 0.02 m): the oracle resumes the GPU world's snapshot after 5
      warm-up steps (the benchmark's) and both step 5 more; pairs, colours, contacts,
      impulses and state bit-exact at every step.
  C2  100,000 mixed spheres / boxes / capsules (20 PGS sweeps): settled on the GPU for 120
      steps, then 4 steps compared the same way.
  C4  the full 4,096-world batch (lognormal body counts, median 256, clipped to [16, 8192])
      stepped 12 steps; 10 sampled worlds, the 3 largest (stepped in the big-world lane)
      among them, bit-exact against single oracle worlds.
  C5  the 2,048-tower scene in tolerance mode (residual 1e-4): settled 5 steps on the GPU,
      then 3 steps compared, sweep counts included.

The oracle runs with every host core.  Integer results (pairs, colours, counts) are exact;
the floating-point results are compared bit for bit (both sides evaluate the same fp32
expressions without contraction), which implies the contract's tolerances.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import axiom_gb300 as ax
import bench

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def oracle_resume(oracle, snap):
    o = ax.PhysicsWorld(ax.default_config(oracle), lib=oracle)
    o.load_snapshot(snap)
    oracle.oracle_set_threads(o.handle, THREADS)
    return o


def pair_keys(w):
    p = w.read_pairs()
    return np.sort(p[:, 0].astype(np.uint64) << np.uint64(32) | p[:, 1].astype(np.uint64))


def same_step(g, o, sg, so, k, contacts=True):
    assert (sg.pair_count, sg.manifold_count, sg.contact_point_count, sg.colour_count, sg.colour_rounds,
            sg.iterations, sg.residual, sg.status, sg.gjk_failures, sg.epa_failures) == \
        (so.pair_count, so.manifold_count, so.contact_point_count, so.colour_count, so.colour_rounds,
         so.iterations, so.residual, so.status, so.gjk_failures, so.epa_failures), k
    assert np.array_equal(pair_keys(g), pair_keys(o)), f"step {k}: pair sets differ"
    if contacts:
        cg = ax.canonical_contacts(g.read_contacts())
        co = ax.canonical_contacts(o.read_contacts())
        for f in ("body_a", "body_b", "point_index", "colour", "position", "normal", "penetration_depth",
                  "impulse"):
            assert np.array_equal(cg[f], co[f]), f"step {k}: {f} differs"
    a, b = g.read_state(), o.read_state()
    for key in a:
        assert np.array_equal(a[key], b[key]), f"step {k}: state {key} differs"


def test_c3_full_pile_five_steps(gpu_lib, oracle):
    sc = bench.pile_scene(gpu_lib)
    g = ax.PhysicsWorld(bench.pile_config(gpu_lib), lib=gpu_lib)
    g.add_bodies(sc.bodies)
    for _ in range(5):
        g.step(bench.DT)
    o = oracle_resume(oracle, g.save_snapshot())
    for k in range(5):
        sg, so = g.step(bench.DT), o.step(bench.DT)
        assert sg.manifold_count > 3_000_000
        same_step(g, o, sg, so, k)


def test_c2_mixed_100k(gpu_lib, oracle):
    sc = ax.Scene.mixed(seed=2, count=100_000, size=(200.0, 100.0, 200.0), lib=gpu_lib)
    cfg = dict(time_step=bench.DT, velocity_iterations=20)
    g = ax.PhysicsWorld(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    g.add_bodies(sc.bodies)
    for _ in range(120):
        g.step(bench.DT, check=False)
    o = oracle_resume(oracle, g.save_snapshot())
    for k in range(4):
        sg, so = g.step(bench.DT, check=False), o.step(bench.DT, check=False)
        assert sg.manifold_count > 1000
        same_step(g, o, sg, so, k)


def test_c4_full_batch_sampled_worlds(gpu_lib, oracle):
    bs = ax.BatchScene(seed=4, worlds=4096, median=256.0, sigma=1.0, min_bodies=16, max_bodies=8192, lib=gpu_lib)
    cfg = dict(time_step=1 / 60, velocity_iterations=10)
    batch = ax.Batch(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    batch.set_worlds(bs.bodies, bs.sizes)
    largest = [int(w) for w in np.argsort(bs.sizes)[-3:]]
    assert bs.sizes[largest].min() >= 4096  # these step in the big-world lane
    check = sorted(set(largest) | {0, 1, 511, 1024, 2047, 3000, 4095})
    worlds = {}
    for w in check:
        o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
        oracle.oracle_set_threads(o.handle, THREADS)
        o.add_bodies(bs.world(w))
        worlds[w] = o
    for step in range(12):
        batch.step(1 / 60, check=False)
        stats = batch.world_stats()
        for w, o in worlds.items():
            so = o.step(1 / 60, check=False)
            assert (stats["pairs"][w], stats["manifolds"][w], stats["colours"][w]) == \
                (so.pair_count, so.manifold_count, so.colour_count), (step, w)
    state = batch.read_state()
    for w, o in worlds.items():
        lo, hi = int(bs.offsets[w]), int(bs.offsets[w + 1])
        so = o.read_state()
        for k in state:
            assert np.array_equal(state[k][lo:hi], so[k]), (w, k)


def test_c5_towers_2048_tolerance_mode(gpu_lib, oracle):
    sc = ax.Scene.towers(seed=5, count=2048, friction=0.6, lib=gpu_lib)
    cfg = dict(time_step=1 / 60, residual_tolerance=1e-4, max_iterations=20000)
    g = ax.PhysicsWorld(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    g.add_bodies(sc.bodies)
    for _ in range(5):
        g.step(1 / 60, check=False)
    o = oracle_resume(oracle, g.save_snapshot())
    for k in range(3):
        sg, so = g.step(1 / 60, check=False), o.step(1 / 60, check=False)
        assert sg.iterations > 100 and sg.residual <= 1e-4
        same_step(g, o, sg, so, k)
