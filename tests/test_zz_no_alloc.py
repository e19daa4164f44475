"""The broadphase entry point that allocates nothing (axiom_broadphase_pairs_static).

Callers that may not allocate device memory at run time (a pre-sized memory pool, a
fixed-rate loop, a plugin whose host owns all allocations) use this entry point; its
scratch is a fixed device array inside the library.  The test feeds it the AABBs the CPU
oracle computed in a step and checks it returns exactly the pair set of the oracle's
broadphase (every pair whose AABBs overlap inclusively with at least one dynamic body;
pairs are integer results: the tolerance is exact equality), on calls in a row with
different inputs, so a call cannot lean on what the previous one left in the shared
scratch: an all-dynamic lattice, a drop of spheres a third of which are static (pairs of
two static bodies are left out), and the same drop with no dynamic flags (all dynamic).
It also checks the size limit, an empty call and a capacity below the pair count.  This
file is collected last so that a failure here stops a run only after every other test
ran.
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


def oracle_pairs(oracle, bodies):
    """Pairs and AABBs from the CPU oracle's broadphase after one step."""
    w = ax.PhysicsWorld(ax.default_config(oracle, time_step=1 / 120), lib=oracle)
    w.add_bodies(bodies)
    w.step(1 / 120)
    mn, mx = w.read_aabbs()
    return ax.canonical_pairs(w.read_pairs()), mn, mx


def all_pairs(mn, mx, dyn):
    """Every (a, b), a < b, with inclusively overlapping AABBs and a dynamic body (numpy)."""
    out = []
    for a in range(len(mn)):
        b = np.arange(a + 1, len(mn))
        hit = np.all((mn[a] <= mx[b]) & (mn[b] <= mx[a]), axis=1) & (dyn[a] | dyn[b])
        out.extend((a, int(x)) for x in b[hit])
    return np.array(sorted(out), np.uint32).reshape(-1, 2)


def static_pairs(fn, torch, mn, mx, dyn, capacity):
    dev = torch.device("cuda", 0)
    tmin = torch.from_numpy(np.ascontiguousarray(mn)).to(dev)
    tmax = torch.from_numpy(np.ascontiguousarray(mx)).to(dev)
    tdyn = None if dyn is None else torch.from_numpy(dyn.astype(np.int32)).to(dev)
    tpairs = torch.zeros(2 * max(capacity, 1), dtype=torch.int32, device=dev)
    tcount = torch.full((1,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    code = fn(tmin.data_ptr(), tmax.data_ptr(), None if tdyn is None else tdyn.data_ptr(), len(mn),
              tpairs.data_ptr(), capacity, tcount.data_ptr(), stream)
    assert code == 0
    torch.cuda.synchronize(dev)
    count = int(tcount.item())
    pairs = tpairs.cpu().numpy().view(np.uint32).reshape(-1, 2)[:min(count, capacity)]
    return count, ax.canonical_pairs(pairs)


def _drop_with_static(lib):
    sc = ax.Scene.sphere_drop(seed=7, count=3000, size=(30.0, 30.0, 30.0), radius=0.6, lib=lib)
    arrays = {k: v.copy() for k, v in sc.bodies.arrays.items()}
    body = arrays["shape"] != ax.SHAPE_PLANE
    arrays["type"][np.nonzero(body)[0][::3]] = ax.BODY_STATIC  # a third of the spheres static
    return ax.Bodies(**arrays)


def test_static_broadphase_matches_oracle(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    fn = bind(gpu_lib)
    lattice = ax.Scene.sphere_lattice(seed=3, dims=(24, 12, 24), lib=gpu_lib).bodies
    drop = _drop_with_static(gpu_lib)
    # calls in a row on the shared scratch: all dynamic, a third static, no flags at all
    for bodies, flags in ((lattice, True), (drop, True), (drop, False)):
        expect, mn, mx = oracle_pairs(oracle, bodies)
        body = bodies.arrays["shape"] != ax.SHAPE_PLANE  # the plane is the last body
        assert body[:-1].all() and not body[-1]
        dyn = bodies.arrays["type"][body] == ax.BODY_DYNAMIC
        if flags:
            assert np.array_equal(expect, all_pairs(mn[body], mx[body], dyn))
            count, got = static_pairs(fn, torch, mn[body], mx[body], dyn, capacity=len(expect) + 64)
            assert count == len(expect)
            assert np.array_equal(got, expect)
        else:
            # no flags: every body dynamic, so the static-static pairs come back too
            want = all_pairs(mn[body], mx[body], np.ones(int(body.sum()), bool))
            assert len(want) > len(expect)
            count, got = static_pairs(fn, torch, mn[body], mx[body], None, capacity=len(want) + 64)
            assert count == len(want)
            assert np.array_equal(got, want)


def test_static_broadphase_limits(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    fn = bind(gpu_lib)
    dev = torch.device("cuda", 0)
    tcount = torch.zeros(1, dtype=torch.int32, device=dev)
    big = torch.zeros(3 * (MAX_BODIES + 1), dtype=torch.float32, device=dev)
    code = fn(big.data_ptr(), big.data_ptr(), None, MAX_BODIES + 1, None, 0, tcount.data_ptr(), None)
    assert code == 600  # InvalidParameter: beyond the fixed scratch
    # no bodies: nothing to sweep, the count is 0
    count, got = static_pairs(fn, torch, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), None, 0)
    assert count == 0 and len(got) == 0
    # capacity smaller than the pair count: the count is still reported in full
    bodies = ax.Scene.sphere_lattice(seed=3, dims=(8, 4, 8), lib=gpu_lib).bodies
    expect, mn, mx = oracle_pairs(oracle, bodies)
    count, got = static_pairs(fn, torch, mn[:-1], mx[:-1], np.ones(len(mn) - 1, bool), capacity=10)
    assert count == len(expect) and len(got) == 10
    assert set(map(tuple, got.tolist())) <= set(map(tuple, expect.tolist()))
