"""Continuous collision by speculative contacts (the reference's design notes ask for CCD
that "prevents tunneling for fast-moving objects", CLAUDE.md:136).

With ``speculative_contacts`` each moving body's AABB is swept by its displacement over the
step and every pair reports a contact while the gap is within the two bodies'
displacements (negative depth): the analytic pairs from their closest points, the
support-mapped pairs (box-box, box-capsule, cylinders, hulls) from GJK + EPA on one shape
inflated by that distance.  The solver lets such a point close exactly its gap.  The
tests fire bodies that move several times their own size per step: without the option they
pass through thin obstacles, with it they stop at the surface.
"""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax

DT = 1.0 / 60.0


def bullet_scene(speed=102.0, r=0.05):
    # a thin static wall (0.1 m thick, x in [1.95, 2.05]) and a small sphere flying at it
    return ax.Bodies(type=[ax.BODY_STATIC, ax.BODY_DYNAMIC], shape=[ax.SHAPE_BOX, ax.SHAPE_SPHERE],
                     position=[(2.0, 0.0, 0.0), (0.0, 0.0, 0.0)], shape_extents=[(0.05, 2.0, 2.0), (r, 0, 0)],
                     linear_velocity=[(0, 0, 0), (speed, 0, 0)], restitution=[0.0, 0.0])


def run(lib, bodies, steps, **cfg):
    c = dict(time_step=DT, velocity_iterations=10, gravity=(0.0, 0.0, 0.0))
    c.update(cfg)
    w = ax.PhysicsWorld(ax.default_config(lib, **c), lib=lib)
    w.add_bodies(bodies)
    trace = []
    for _ in range(steps):
        st = w.step(DT)
        trace.append((w.read_state(), st))
    return w, trace


def test_oracle_bullet_tunnels_without_and_stops_with_ccd(oracle):
    _, off = run(oracle, bullet_scene(), 6)
    assert off[-1][0]["position"][1, 0] > 2.1  # 1.7 m per step: from 0.2 m short of the wall to past it
    _, on = run(oracle, bullet_scene(), 6, speculative_contacts=1)
    x = np.array([s["position"][1, 0] for s, _ in on])
    assert x.max() < 1.95 - 0.05 + 1e-3  # never past the wall's near face (minus its radius)
    assert abs(on[-1][0]["linear_velocity"][1, 0]) < 1e-3  # stopped (no restitution)
    assert min(st.manifold_count for _, st in on) >= 0 and max(st.manifold_count for _, st in on) == 1


def thin_box_scene(shape, speed=102.0):
    # a thin static box wall (x in [1.95, 2.05]) and a fast body of the given shape: a box
    # 0.1 m thick in x, or a capsule / cylinder lying along x... standing along y, 0.05 m
    # in radius, either way much thinner than its 1.7 m displacement per step
    ext = {ax.SHAPE_BOX: (0.05, 0.3, 0.3), ax.SHAPE_CAPSULE: (0.05, 0.3, 0.0),
           ax.SHAPE_CYLINDER: (0.05, 0.3, 0.0)}[shape]
    return ax.Bodies(type=[ax.BODY_STATIC, ax.BODY_DYNAMIC], shape=[ax.SHAPE_BOX, shape],
                     position=[(2.0, 0.0, 0.0), (0.0, 0.0, 0.0)], shape_extents=[(0.05, 2.0, 2.0), ext],
                     linear_velocity=[(0, 0, 0), (speed, 0, 0)], restitution=[0.0, 0.0])


@pytest.mark.parametrize("shape", [ax.SHAPE_BOX, ax.SHAPE_CAPSULE, ax.SHAPE_CYLINDER])
def test_oracle_fast_thin_body_stops_at_thin_box(oracle, shape):
    """Support-mapped pairs (GJK): a thin box, capsule or cylinder fired at a thin box wall
    passes through it without CCD and stops at its face with it."""
    _, off = run(oracle, thin_box_scene(shape), 6)
    assert off[-1][0]["position"][1, 0] > 2.1
    _, on = run(oracle, thin_box_scene(shape), 6, speculative_contacts=1)
    x = np.array([s["position"][1, 0] for s, _ in on])
    assert x.max() < 1.95 - 0.05 + 2e-3  # never past the wall's near face
    assert abs(on[-1][0]["linear_velocity"][1, 0]) < 1e-2  # stopped (no restitution)
    assert any(st.manifold_count == 1 for _, st in on)


def test_oracle_fast_sphere_hits_resting_sphere(oracle):
    # a 0.1 m sphere at 60 m/s (1 m per step) towards a resting one 3.5 m away: the plain step
    # goes from 0.3 m short of it (x = 3) to 0.3 m past it (x = 4)
    b = ax.Bodies(type=[1, 1], shape=[0, 0], position=[(0, 0, 0), (3.5, 0, 0)], shape_extents=[(0.1, 0, 0)] * 2,
                  linear_velocity=[(60.0, 0, 0), (0, 0, 0)], restitution=[0.0, 0.0])
    _, off = run(oracle, b, 8)
    assert np.abs(off[-1][0]["linear_velocity"][1]).max() == 0.0  # missed it entirely
    _, on = run(oracle, b, 8, speculative_contacts=1)
    v = on[-1][0]["linear_velocity"]
    assert v[1, 0] > 20.0  # momentum went into the target
    assert on[-1][0]["position"][0, 0] < on[-1][0]["position"][1, 0]  # still on its own side


def test_oracle_fast_box_lands_on_ground_without_deep_penetration(oracle):
    b = ax.Bodies(type=[0, 1], shape=[ax.SHAPE_PLANE, ax.SHAPE_BOX], position=[(0, 0, 0), (0, 3.3, 0)],
                  shape_extents=[(0, 0, 0), (0.5, 0.5, 0.5)], linear_velocity=[(0, 0, 0), (0, -50.0, 0)],
                  restitution=[0.0, 0.0])
    deepest = {}
    for spec in (0, 1):
        _, trace = run(oracle, b, 12, speculative_contacts=spec, gravity=(0, -9.81, 0))
        ys = [s["position"][1, 1] for s, _ in trace]
        deepest[spec] = 0.5 - min(ys)
    assert deepest[0] > 0.3      # plain: the box sinks most of the way in before it is pushed out
    assert deepest[1] < 0.02     # swept: it stops at the ground


def test_ccd_off_by_default(oracle):
    w = ax.PhysicsWorld(ax.default_config(oracle), lib=oracle)
    assert w.config.speculative_contacts == 0


@pytest.mark.gpu
def test_gpu_ccd_bit_exact(gpu_lib, oracle):
    # a pile of mixed shapes on the ground, bombarded by fast spheres and capsules
    rng = np.random.default_rng(5)
    n = 300
    shapes = rng.choice([ax.SHAPE_SPHERE, ax.SHAPE_BOX, ax.SHAPE_CAPSULE, ax.SHAPE_CYLINDER], n)
    k = np.arange(n)
    pos = np.column_stack([(k % 10) * 1.2, 0.6 + (k // 100) * 1.2, ((k // 10) % 10) * 1.2]) + rng.uniform(-0.05, 0.05, (n, 3))
    vel = np.zeros((n, 3))
    fast = rng.random(n) < 0.15
    vel[fast] = rng.normal(size=(fast.sum(), 3)) * 40.0
    ext = np.column_stack([rng.uniform(0.2, 0.4, n), rng.uniform(0.2, 0.4, n), rng.uniform(0.2, 0.4, n)])
    b = ax.Bodies(type=np.r_[0, np.ones(n)].astype(np.uint32), shape=np.r_[ax.SHAPE_PLANE, shapes].astype(np.uint32),
                  position=np.vstack([[0, 0, 0], pos]), shape_extents=np.vstack([[0, 0, 0], ext]),
                  linear_velocity=np.vstack([[0, 0, 0], vel]), friction=np.full(n + 1, 0.5))
    cfg = dict(time_step=1 / 120, velocity_iterations=10, speculative_contacts=1)
    g = ax.PhysicsWorld(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    oracle.oracle_set_threads(o.handle, 8)
    g.add_bodies(b)
    o.add_bodies(b)
    negative = 0
    for step in range(120):
        sg, so = g.step(1 / 120), o.step(1 / 120)
        assert (sg.pair_count, sg.manifold_count, sg.contact_point_count) == \
            (so.pair_count, so.manifold_count, so.contact_point_count), step
        a, c = g.read_state(), o.read_state()
        for key in a:
            assert np.array_equal(a[key], c[key]), (step, key)
        if step % 20 == 0:
            cg = ax.canonical_contacts(g.read_contacts())
            co = ax.canonical_contacts(o.read_contacts())
            assert cg.tobytes() == co.tobytes(), step
            negative += int((cg["penetration_depth"] < 0).sum())
    assert negative > 0  # speculative (separated) contacts were exercised


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [ax.SHAPE_BOX, ax.SHAPE_CAPSULE, ax.SHAPE_CYLINDER])
def test_gpu_fast_thin_body_bit_exact(gpu_lib, oracle, shape):
    _, g = run(gpu_lib, thin_box_scene(shape), 6, speculative_contacts=1)
    _, o = run(oracle, thin_box_scene(shape), 6, speculative_contacts=1)
    for (sg, stg), (so, sto) in zip(g, o):
        assert stg.manifold_count == sto.manifold_count
        for key in sg:
            assert np.array_equal(sg[key], so[key]), key
    assert g[-1][0]["position"][1, 0] < 1.9 + 2e-3


@pytest.mark.gpu
def test_gpu_bullet_stops(gpu_lib):
    _, on = run(gpu_lib, bullet_scene(), 6, speculative_contacts=1)
    x = np.array([s["position"][1, 0] for s, _ in on])
    assert x.max() < 1.9 + 1e-3
