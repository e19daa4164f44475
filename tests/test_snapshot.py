"""World snapshot / resume and the headless debug feed.

A snapshot (layout in include/axiom_c.h) holds the configuration, every body and the
previous-step warm-start impulses; a world loaded from it must continue bit for bit as
the original does.  The GPU library and the CPU oracle share the byte format, so the GPU
tests also check that both write identical bytes for identical worlds and that each
resumes the other's snapshot.  The debug feed carries the records of
debug::PhysicsDebugDraw (include/axiom/debug/physics_debug_draw.hpp:97-132).
"""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax

DT = 1.0 / 120.0


def mixed_scene(lib, count=600, seed=11):
    sc = ax.Scene.mixed(seed=seed, count=count, size=(10.0, 14.0, 10.0), lib=lib)
    n = sc.bodies.n
    rng = np.random.default_rng(seed)
    arrays = dict(sc.bodies.arrays)
    # some non-default filters and a few bodies that may not sleep, so every record field varies
    arrays["filter_group"] = rng.choice(np.array([0, 0, 0, 1, -1], np.int16), n)
    arrays["allow_sleep"] = (rng.random(n) > 0.1).astype(np.uint8)
    return ax.Bodies(**arrays)


def world(lib, bodies, **cfg):
    c = dict(time_step=DT, velocity_iterations=8, allow_sleep=1, sleep_linear_threshold=0.05,
             sleep_angular_threshold=0.1, sleep_time_threshold=0.1)
    c.update(cfg)
    w = ax.PhysicsWorld(ax.default_config(lib, **c), lib=lib)
    if bodies is not None:
        w.add_bodies(bodies)
    return w


def states_equal(a, b):
    sa, sb = a.read_state(), b.read_state()
    return all(np.array_equal(sa[k], sb[k]) for k in sa)


# ---------------------------------------------------------------- oracle (CPU) ----

def test_oracle_snapshot_resumes_bit_exact(lib, oracle):
    b = mixed_scene(lib)
    w = world(oracle, b)
    for _ in range(40):
        w.step(DT)
    snap = w.save_snapshot()
    for _ in range(25):
        w.step(DT)
    r = world(oracle, None)
    r.load_snapshot(snap)
    assert r.body_count() == b.n
    assert r.save_snapshot() == snap  # load then save is the identity
    for _ in range(25):
        r.step(DT)
    assert states_equal(w, r)
    assert np.array_equal(w.read_sleep()["sleeping"], r.read_sleep()["sleeping"])
    assert w.save_snapshot() == r.save_snapshot()


def test_oracle_snapshot_layout(lib, oracle):
    b = mixed_scene(lib)
    w = world(oracle, b)
    for _ in range(10):
        st = w.step(DT)
    snap = w.save_snapshot()
    h, bodies, warm, hulls = ax.parse_snapshot(snap)
    assert h.magic == b"AXSNAP01" and h.version == 3 and h.flags == 1 and hulls == []
    assert h.body_count == b.n and h.total_bytes == len(snap)
    assert h.config.allow_sleep == 1 and h.config.time_step == pytest.approx(DT)
    s = w.read_state()
    assert np.array_equal(bodies["position"], s["position"])
    assert np.array_equal(bodies["rotation"], s["rotation"])
    assert np.array_equal(bodies["linear_velocity"], s["linear_velocity"])
    assert np.array_equal(bodies["type"], b.arrays["type"])
    assert np.array_equal(bodies["filter_group"], b.arrays["filter_group"].astype(np.int32))
    # one entry per contact point of the last step, sorted by (lo, hi, point); point 0 of a
    # manifold carries 1 + its colour in bits 8-15
    assert len(warm) == st.contact_point_count
    point = warm["point"] & 0xFF
    keys = (warm["body_lo"].astype(np.uint64) << np.uint64(34)) | (warm["body_hi"].astype(np.uint64) << np.uint64(2)) \
        | point.astype(np.uint64)
    assert np.all(np.diff(keys.astype(np.float64)) > 0)
    c0 = ax.canonical_contacts(w.read_contacts())
    c0 = c0[c0["point_index"] == 0]
    lo0, hi0 = np.minimum(c0["body_a"], c0["body_b"]), np.maximum(c0["body_a"], c0["body_b"])
    tag = dict(zip(zip(warm["body_lo"][point == 0].tolist(), warm["body_hi"][point == 0].tolist()),
                   (warm["point"][point == 0] >> 8).tolist()))
    assert all(tag[(int(a), int(b))] == int(col) + 1 for a, b, col in zip(lo0, hi0, c0["colour"]))
    assert (warm["point"][point > 0] >> 8 == 0).all()
    c = ax.canonical_contacts(w.read_contacts())
    lo = np.minimum(c["body_a"], c["body_b"])
    hi = np.maximum(c["body_a"], c["body_b"])
    order = np.lexsort((c["point_index"], hi, lo))
    assert np.array_equal(warm["impulse"], c["impulse"][order])


def test_load_rejects_malformed_snapshots(lib, oracle):
    b = mixed_scene(lib, count=50)
    w = world(oracle, b)
    w.step(DT)
    snap = bytearray(w.save_snapshot())
    r = world(oracle, None)
    for bad in (snap[:-4], b"XXSNAP01" + snap[8:], snap[:100]):
        with pytest.raises(ax.AxiomError) as e:
            r.load_snapshot(bytes(bad))
        assert e.value.code == 600
    hs = ax.ctypes.sizeof(ax.SnapshotHeader)
    hdr = ax.SnapshotHeader.from_buffer_copy(bytes(snap[:hs]))
    bad = bytearray(snap)
    bad[hs:hs + 4] = (7).to_bytes(4, "little")  # first body's type
    with pytest.raises(ax.AxiomError):
        r.load_snapshot(bytes(bad))
    assert hdr.body_count == b.n


def test_oracle_debug_feed(lib, oracle):
    b = mixed_scene(lib, count=300)
    w = world(oracle, b)
    for _ in range(30):
        w.step(DT)
    bodies, contacts = w.read_debug(ax.DEBUG_ALL)
    s = w.read_state()
    mn, mx = w.read_aabbs()
    sl = w.read_sleep()
    assert np.array_equal(bodies["position"], s["position"]) and np.array_equal(bodies["rotation"], s["rotation"])
    assert np.array_equal(bodies["aabb_min"], mn) and np.array_equal(bodies["aabb_max"], mx)
    assert np.array_equal(bodies["linear_velocity"], s["linear_velocity"])
    assert np.array_equal(bodies["shape"], b.arrays["shape"])
    assert np.array_equal(bodies["island_index"], sl["island"])
    dyn = b.arrays["type"] == ax.BODY_DYNAMIC
    assert np.array_equal(bodies["is_awake"][dyn], (sl["sleeping"][dyn] == 0).astype(np.uint32))
    c = w.read_contacts()
    assert len(contacts) == len(c)
    # unselected sections stay zero
    only, none = w.read_debug(ax.DEBUG_SHAPES)
    assert len(none) == 0 and not only["aabb_min"].any() and not only["linear_velocity"].any()
    assert np.array_equal(only["position"], s["position"])


# ------------------------------------------------------------ GPU vs oracle ----

def debug_sorted(c):
    return c[np.lexsort((c["position"][:, 2], c["position"][:, 1], c["position"][:, 0], c["body_b"], c["body_a"]))]


@pytest.mark.gpu
def test_gpu_snapshot_bytes_equal_oracle_and_cross_resume(gpu_lib, oracle):
    b = mixed_scene(gpu_lib, count=2000)
    g, o = world(gpu_lib, b), world(oracle, b)
    oracle.oracle_set_threads(o.handle, 8)
    for _ in range(60):
        g.step(DT)
        o.step(DT)
    sg, so = g.save_snapshot(), o.save_snapshot()
    assert sg == so  # same world, same bytes
    # each implementation resumes the other's snapshot
    g2, o2 = world(gpu_lib, None), world(oracle, None)
    g2.load_snapshot(so)
    o2.load_snapshot(sg)
    oracle.oracle_set_threads(o2.handle, 8)
    for k in range(40):
        for w in (g, o, g2, o2):
            w.step(DT)
        assert states_equal(g, g2) and states_equal(o, o2) and states_equal(g, o), k
    assert g.save_snapshot() == g2.save_snapshot() == o2.save_snapshot()


@pytest.mark.gpu
def test_gpu_debug_feed_equals_oracle(gpu_lib, oracle):
    b = mixed_scene(gpu_lib, count=2000)
    g, o = world(gpu_lib, b), world(oracle, b)
    for _ in range(30):
        g.step(DT)
        o.step(DT)
    bg, cg = g.read_debug()
    bo, co = o.read_debug()
    assert bg.tobytes() == bo.tobytes()
    assert len(cg) == len(co) > 0
    assert debug_sorted(cg).tobytes() == debug_sorted(co).tobytes()


@pytest.mark.gpu
def test_gpu_snapshot_large_pile_resume(gpu_lib):
    # 262,145 bodies: the snapshot path at scale (records packed on the device)
    sc = ax.Scene.sphere_lattice(seed=3, dims=(128, 16, 128), lib=gpu_lib)
    cfg = dict(time_step=DT, velocity_iterations=10)
    w = ax.PhysicsWorld(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    w.add_bodies(sc.bodies)
    for _ in range(3):
        w.step(DT)
    snap = w.save_snapshot()
    h, _, warm, _ = ax.parse_snapshot(snap)
    assert h.body_count == sc.bodies.n and len(warm) > 700_000
    r = ax.PhysicsWorld(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    r.load_snapshot(snap)
    for _ in range(3):
        w.step(DT)
        r.step(DT)
    assert states_equal(w, r)
