"""The broadphase entry point that allocates nothing (axiom_broadphase_pairs_static).

Callers that may not allocate device memory at run time (a pre-sized memory pool, a
fixed-rate loop, a plugin whose host owns all allocations) use this entry point; its
scratch is a fixed device array inside the library.  The test feeds it the AABBs a world
computed in its last step and checks it returns exactly the pair set that world's
broadphase produced (pairs are integer results: the tolerance is exact equality), on
two calls in a row with different inputs, so a call cannot lean on what the previous one
left in the shared scratch.  It also checks the size limit is enforced.  This file is
collected last so that a failure here stops a run only after every other test ran.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import axiom_gb300 as ax

pytestmark = pytest.mark.gpu

MAX_BODIES = 65536


def bind(lib):
    fn = lib.axiom_broadphase_pairs_static
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                   ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
    return fn


def world_pairs(lib, scene):
    """Pairs and AABBs from the world's own broadphase (the allocating entry point)."""
    w = ax.PhysicsWorld(ax.default_config(lib, time_step=1 / 120), lib=lib)
    w.add_bodies(scene.bodies)
    w.step(1 / 120)
    mn, mx = w.read_aabbs()
    return ax.canonical_pairs(w.read_pairs()), mn, mx


def static_pairs(fn, torch, mn, mx, dyn, capacity):
    dev = torch.device("cuda", 0)
    tmin = torch.from_numpy(np.ascontiguousarray(mn)).to(dev)
    tmax = torch.from_numpy(np.ascontiguousarray(mx)).to(dev)
    tdyn = torch.from_numpy(dyn.astype(np.int32)).to(dev)
    tpairs = torch.zeros(2 * capacity, dtype=torch.int32, device=dev)
    tcount = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    code = fn(tmin.data_ptr(), tmax.data_ptr(), tdyn.data_ptr(), len(mn), tpairs.data_ptr(),
              capacity, tcount.data_ptr(), stream)
    assert code == 0
    torch.cuda.synchronize(dev)
    count = int(tcount.item())
    pairs = tpairs.cpu().numpy().view(np.uint32).reshape(-1, 2)[:min(count, capacity)]
    return count, ax.canonical_pairs(pairs)


def test_static_broadphase_matches_world(gpu_lib):
    torch = pytest.importorskip("torch")
    fn = bind(gpu_lib)
    scenes = [ax.Scene.sphere_lattice(seed=3, dims=(24, 12, 24), lib=gpu_lib),
              ax.Scene.sphere_drop(seed=7, count=3000, size=(30.0, 30.0, 30.0), radius=0.6, lib=gpu_lib)]
    for scene in scenes:  # two calls in a row on the shared scratch
        expect, mn, mx = world_pairs(gpu_lib, scene)
        body = scene.bodies.arrays["shape"] != ax.SHAPE_PLANE  # the plane is the last body
        assert body[:-1].all() and not body[-1]
        dyn = scene.bodies.arrays["type"][body] == ax.BODY_DYNAMIC
        count, got = static_pairs(fn, torch, mn[body], mx[body], dyn, capacity=len(expect) + 64)
        assert count == len(expect)
        assert np.array_equal(got, expect)


def test_static_broadphase_limits(gpu_lib):
    torch = pytest.importorskip("torch")
    fn = bind(gpu_lib)
    dev = torch.device("cuda", 0)
    tcount = torch.zeros(1, dtype=torch.int32, device=dev)
    big = torch.zeros(3 * (MAX_BODIES + 1), dtype=torch.float32, device=dev)
    code = fn(big.data_ptr(), big.data_ptr(), None, MAX_BODIES + 1, None, 0, tcount.data_ptr(), None)
    assert code == 600  # InvalidParameter: beyond the fixed scratch
    # capacity smaller than the pair count: the count is still reported in full
    scene = ax.Scene.sphere_lattice(seed=3, dims=(8, 4, 8), lib=gpu_lib)
    expect, mn, mx = world_pairs(gpu_lib, scene)
    count, got = static_pairs(fn, torch, mn[:-1], mx[:-1], np.ones(len(mn) - 1, bool), capacity=10)
    assert count == len(expect) and len(got) == 10
    assert set(map(tuple, got.tolist())) <= set(map(tuple, expect.tolist()))
