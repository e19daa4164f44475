"""Broadphase with bodies of very different sizes.

The uniform grid needs cells as wide as its widest body, so one huge body (a 200 m static
box under a pile of 0.5 m spheres, a large mesh triangle) would put everything into a few
huge cells and make the sweep quadratic.  Bodies wider than 8 x the median width (at most
64 of them) therefore stay out of the grid and are tested against every body.  The pair
set does not change: the tests check it against a brute-force pair test (CPU, oracle) and
the GPU against the oracle bit for bit, on 100,000 spheres resting on one 200 m box.
"""
from __future__ import annotations

import time

import numpy as np
import pytest

import axiom_gb300 as ax

DT = 1.0 / 120.0


def pile_on_slab(nx, ny, nz, spacing=0.52, r=0.25, seed=0):
    """nx*ny*nz spheres on a jittered lattice just above a 200 m x 2 m x 200 m static box."""
    rng = np.random.default_rng(seed)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    pos = np.column_stack([(i.ravel() - nx / 2) * spacing, 1.0 + r + j.ravel() * spacing,
                           (k.ravel() - nz / 2) * spacing]).astype(np.float32)
    pos += rng.uniform(-0.002, 0.002, pos.shape).astype(np.float32)
    n = len(pos)
    return ax.Bodies(type=np.r_[np.ones(n), 0].astype(np.uint32),
                     shape=np.r_[np.full(n, ax.SHAPE_SPHERE), ax.SHAPE_BOX].astype(np.uint32),
                     position=np.vstack([pos, [[0.0, 0.0, 0.0]]]),
                     shape_extents=np.vstack([np.tile([r, 0, 0], (n, 1)), [[100.0, 1.0, 100.0]]]).astype(np.float32),
                     friction=np.full(n + 1, 0.5, np.float32), restitution=np.zeros(n + 1, np.float32))


def brute_pairs(mn, mx, dyn):
    out = []
    for a in range(len(mn)):
        b = np.arange(a + 1, len(mn))
        hit = np.all((mn[a] <= mx[b]) & (mn[b] <= mx[a]), axis=1) & (dyn[a] | dyn[b])
        out.extend((a, int(x)) for x in b[hit])
    return np.array(sorted(out), np.uint32).reshape(-1, 2)


def test_oracle_pairs_with_a_huge_box(oracle):
    b = pile_on_slab(20, 3, 20)
    w = ax.PhysicsWorld(ax.default_config(oracle, time_step=DT), lib=oracle)
    w.add_bodies(b)
    for _ in range(3):
        w.step(DT)
    mn, mx = w.read_aabbs()
    dyn = b.arrays["type"] == ax.BODY_DYNAMIC
    got = ax.canonical_pairs(w.read_pairs())
    assert np.array_equal(got, brute_pairs(mn, mx, dyn))
    assert (got[:, 1] == b.n - 1).sum() == 400  # the bottom layer touches the slab


@pytest.mark.gpu
def test_gpu_100k_spheres_on_a_200m_box_bit_exact(gpu_lib, oracle):
    import os

    b = pile_on_slab(100, 10, 100)
    cfg = dict(time_step=DT, velocity_iterations=10)
    g = ax.PhysicsWorld(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    oracle.oracle_set_threads(o.handle, os.cpu_count() or 1)
    g.add_bodies(b)
    o.add_bodies(b)
    ms = []
    for k in range(5):
        t0 = time.perf_counter()
        sg = g.step(DT)
        ms.append((time.perf_counter() - t0) * 1e3)
        so = o.step(DT)
        assert (sg.pair_count, sg.manifold_count, sg.colour_count) == (so.pair_count, so.manifold_count,
                                                                       so.colour_count), k
        assert np.array_equal(ax.canonical_pairs(g.read_pairs()), ax.canonical_pairs(o.read_pairs())), k
        a, c = g.read_state(), o.read_state()
        for key in a:
            assert np.array_equal(a[key], c[key]), (k, key)
    assert sg.manifold_count >= 10_000  # every sphere of the bottom layer on the box
    # without the large-body path this step sweeps 100,000 bodies in one 200 m cell
    assert min(ms) < 50.0, ms
