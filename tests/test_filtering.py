"""Collision filtering (gui::FilterInfo, include/axiom/gui/body_inspector.hpp:38-42).

Two bodies with the same non-zero group always (group > 0) or never (group < 0) collide;
otherwise they collide when each one's category is in the other's mask.  Defaults:
category 0x0001, mask 0xFFFF, group 0.  Filtering removes pairs in the broadphase and
body-plane contacts; everything downstream sees only the surviving pairs.
"""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax


def should_collide(cat, msk, grp, a, b):
    if grp[a] == grp[b] and grp[a] != 0:
        return grp[a] > 0
    return bool(msk[a] & cat[b]) and bool(cat[a] & msk[b])


def filtered_scene(lib, seed=2, count=3000):
    sc = ax.Scene.mixed(seed=seed, count=count, size=(20.0, 24.0, 20.0), lib=lib)
    rng = np.random.default_rng(seed)
    n = sc.bodies.n
    cat = rng.choice(np.array([1, 2, 4, 8], np.uint32), n)
    msk = rng.choice(np.array([0xFFFF, 0xFFFF, 0x000F, 0x0003, 0x000C, 0x0005], np.uint32), n)
    grp = rng.choice(np.array([0, 0, 0, 0, 1, -1, 2, -2], np.int16), n)
    # the ground plane (last body) keeps a filter that some bodies reject
    cat[-1], msk[-1], grp[-1] = 1, 0xFFFF, 0
    arrays = dict(sc.bodies.arrays)
    arrays.update(filter_category=cat, filter_mask=msk, filter_group=grp)
    return sc.bodies, ax.Bodies(**arrays), (cat, msk, grp)


def test_filter_defaults_collide_everything(oracle):
    # default filters (category 1, mask 0xFFFF, group 0) pass every pair
    cat = np.array([1, 1], np.uint32)
    msk = np.array([0xFFFF, 0xFFFF], np.uint32)
    grp = np.array([0, 0], np.int16)
    assert should_collide(cat, msk, grp, 0, 1)


def test_oracle_drops_rejected_pairs_and_plane_contacts(lib, oracle):
    plain, filt, (cat, msk, grp) = filtered_scene(lib)
    cfg = dict(time_step=1 / 120, velocity_iterations=4)
    w0 = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    w1 = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    w0.add_bodies(plain)
    w1.add_bodies(filt)
    w0.step(1 / 120)
    w1.step(1 / 120)
    p0 = ax.canonical_pairs(w0.read_pairs())
    p1 = ax.canonical_pairs(w1.read_pairs())
    keep = np.array([should_collide(cat, msk, grp, a, b) for a, b in p0], bool)
    assert 0 < keep.sum() < len(p0)  # the filters remove some pairs, not all
    assert np.array_equal(p1, p0[keep])


def test_oracle_filters_plane_contacts(lib, oracle):
    # a resting lattice: the whole bottom layer touches the ground plane at the first step
    sc = ax.Scene.sphere_lattice(seed=3, dims=(10, 2, 10), lib=lib)
    n = sc.bodies.n
    rng = np.random.default_rng(1)
    cat = rng.choice(np.array([1, 2], np.uint32), n)
    msk = rng.choice(np.array([0xFFFF, 0x0002], np.uint32), n)
    grp = rng.choice(np.array([0, 0, -3], np.int16), n)
    plane = n - 1
    cat[plane], msk[plane], grp[plane] = 1, 0xFFFF, -3
    arrays = dict(sc.bodies.arrays)
    arrays.update(filter_category=cat, filter_mask=msk, filter_group=grp)
    touching = []
    for bodies in (sc.bodies, ax.Bodies(**arrays)):
        w = ax.PhysicsWorld(ax.default_config(oracle, time_step=1 / 120), lib=oracle)
        w.add_bodies(bodies)
        w.step(1 / 120)
        c = w.read_contacts()
        touching.append(set(c["body_b"][c["body_a"] == plane].tolist()))
    expect = {i for i in touching[0] if should_collide(cat, msk, grp, plane, i)}
    assert expect and len(expect) < len(touching[0])
    assert touching[1] == expect


@pytest.mark.gpu
def test_gpu_filtering_matches_oracle(gpu_lib, oracle):
    _, filt, _ = filtered_scene(gpu_lib)
    cfg = dict(time_step=1 / 120, velocity_iterations=10)
    g = ax.PhysicsWorld(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    g.add_bodies(filt)
    o.add_bodies(filt)
    for k in range(30):
        g.step(1 / 120)
        o.step(1 / 120)
        assert np.array_equal(ax.canonical_pairs(g.read_pairs()), ax.canonical_pairs(o.read_pairs())), k
        cg = ax.canonical_contacts(g.read_contacts())
        co = ax.canonical_contacts(o.read_contacts())
        assert np.array_equal(cg, co), k
    sg, so = g.read_state(), o.read_state()
    for key in sg:
        assert np.array_equal(sg[key], so[key]), key


@pytest.mark.gpu
def test_batch_filtering_matches_oracle(gpu_lib, oracle):
    _, filt, _ = filtered_scene(gpu_lib, seed=5, count=300)
    cfg = dict(time_step=1 / 60, velocity_iterations=10)
    # the same filtered world twice in one batch
    arrays = {k: np.concatenate([v, v]) for k, v in filt.arrays.items()}
    batch = ax.Batch(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    batch.set_worlds(ax.Bodies(**arrays), np.array([filt.n, filt.n], np.uint32))
    o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    o.add_bodies(filt)
    for _ in range(20):
        batch.step(1 / 60)
        so = o.step(1 / 60)
        st = batch.world_stats()
        assert st["pairs"][0] == so.pair_count and st["pairs"][1] == so.pair_count
    state = batch.read_state()
    ref = o.read_state()
    for key in state:
        assert np.array_equal(state[key][: filt.n], ref[key]), key
        assert np.array_equal(state[key][filt.n:], ref[key]), key
