"""Sleeping and islands (PhysicsWorldConfig::allowSleep and thresholds,
include/axiom/gui/physics_panel.hpp:39-42; per-body gui::SleepInfo,
include/axiom/gui/body_inspector.hpp:45-51; PhysicsWorldStats::islandCount and
sleepingBodies, physics_panel.hpp:13-23).

Rules under test: an island (dynamic bodies linked by contacts between two awake dynamic
bodies) falls asleep once every body in it has stayed at or below both velocity thresholds
for sleep_time_threshold; it is labelled by its lowest body id; a sleeping island wakes in
the same step in which an awake dynamic or a moving kinematic body touches it, and the
step's contacts are then computed with it awake.  CPU tests run the oracle; GPU tests
compare the CUDA step with it bit for bit, sleep state included.
"""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax

DT = 1.0 / 60.0
H = 0.5  # box half-extent
NX = NZ = 4


def stacks(nx=NX, nz=NZ):
    """Ground plane + an nx x nz grid of separate box stacks, 1-3 boxes high."""
    t, s, p, e = [ax.BODY_STATIC], [ax.SHAPE_PLANE], [(0.0, 0.0, 0.0)], [(0.0, 0.0, 0.0)]
    for i in range(nx):
        for j in range(nz):
            for k in range(1 + (i + j) % 3):
                t.append(ax.BODY_DYNAMIC)
                s.append(ax.SHAPE_BOX)
                p.append((i * 2.0, H + k * (2 * H - 0.004), j * 2.0))
                e.append((H, H, H))
    return ax.Bodies(type=t, shape=s, position=p, shape_extents=e, friction=[0.6] * len(t))


DEFAULTS = {"linear_velocity": (0.0, 0.0, 0.0), "friction": 0.5, "allow_sleep": 1, "is_sleeping": 0}


def concat(*parts):
    """One body description from several, filling fields some parts lack with defaults."""
    names = set().union(*(p.arrays for p in parts))
    out = {}
    for name in names:
        cols = []
        for p in parts:
            if name in p.arrays:
                cols.append(p.arrays[name])
            else:
                cols.append(np.array([DEFAULTS[name]] * p.n, dtype=parts[0].arrays.get(name, p.arrays["position"]).dtype
                                     if name not in ("allow_sleep", "is_sleeping") else np.uint8))
        out[name] = np.concatenate(cols)
    return ax.Bodies(**out)


def stack_labels(bodies):
    """Expected island label (lowest body id of the stack) of every box."""
    pos = bodies.arrays["position"]
    labels = np.full(bodies.n, 0xFFFFFFFF, np.uint32)
    first = {}
    for i in range(1, bodies.n):
        key = (round(float(pos[i, 0]), 3), round(float(pos[i, 2]), 3))
        first.setdefault(key, i)
        labels[i] = first[key]
    return labels


def world(lib, bodies, **cfg):
    c = dict(time_step=DT, velocity_iterations=10, allow_sleep=1)
    c.update(cfg)
    w = ax.PhysicsWorld(ax.default_config(lib, **c), lib=lib)
    w.add_bodies(bodies)
    return w


def settle(w, max_steps=150):
    for k in range(max_steps):
        st = w.step(DT)
        if st.sleeping_bodies == st.dynamic_bodies:
            return k, st
    raise AssertionError("the stacks never fell asleep")


# ---------------------------------------------------------------- oracle (CPU) ----

def test_oracle_stacks_fall_asleep_as_islands(oracle):
    b = stacks()
    w = world(oracle, b)
    st = w.step(DT)
    assert st.island_count == NX * NZ  # each stack one island; the plane links nothing
    k, st = settle(w)
    assert k >= int(0.5 / DT) - 1  # not before sleep_time_threshold of rest
    sl = w.read_sleep()
    assert sl["sleeping"][1:].all() and not sl["sleeping"][0]
    assert np.array_equal(sl["island"], stack_labels(b))
    assert (sl["sleep_time"][1:] >= 0.5).all()
    before = w.read_state()
    for _ in range(5):
        st = w.step(DT)
        assert st.manifold_count == 0 and st.pair_count == 0 and st.island_count == 0
        assert st.active_bodies == 0 and st.sleeping_bodies == b.n - 1
    after = w.read_state()
    for key in before:
        assert np.array_equal(before[key], after[key]), key  # sleeping bodies do not move
    assert not np.any(after["linear_velocity"]) and not np.any(after["angular_velocity"])


def drop_on_tallest(w, b):
    """Adds a sphere above the first 3-box stack; returns (its id, the stack's ids)."""
    labels = stack_labels(b)
    counts = np.bincount(labels[1:])
    label = int(np.flatnonzero(counts == 3)[0])
    ids = np.flatnonzero(labels == label)
    x, z = b.arrays["position"][label, [0, 2]]
    sid = w.add_bodies(ax.Bodies(type=[ax.BODY_DYNAMIC], shape=[ax.SHAPE_SPHERE],
                                 position=[(float(x), 4.0, float(z))], shape_extents=[(0.3, 0.0, 0.0)]))
    return sid, ids


def test_oracle_contact_wakes_the_whole_island_in_that_step(oracle):
    b = stacks()
    w = world(oracle, b)
    settle(w)
    sid, ids = drop_on_tallest(w, b)
    asleep0 = b.n - 1
    for k in range(120):
        st = w.step(DT)
        if st.manifold_count:
            break
    else:
        raise AssertionError("the sphere never reached the stack")
    # the contact step: the stack woke and its contacts were computed with it awake
    assert st.sleeping_bodies == asleep0 - len(ids)
    sl = w.read_sleep()
    assert not sl["sleeping"][ids].any() and not sl["sleeping"][sid]
    assert st.manifold_count >= len(ids) + 1  # sphere-box, box-box stack contacts, box-plane
    c = w.read_contacts()
    touched = set(c["body_a"]) | set(c["body_b"])
    assert set(ids.tolist()) <= touched and sid in touched
    others = np.setdiff1d(np.arange(1, b.n), ids)
    assert sl["sleeping"][others].all()  # other islands sleep on


def test_oracle_set_sleeping_api(oracle):
    b = stacks()
    w = world(oracle, b)
    settle(w)
    w.set_sleeping([1], False)
    assert w.read_sleep()["sleeping"][1] == 0
    st = w.step(DT)
    # the woken box touches the rest of its island (if any) and wakes it
    labels = stack_labels(b)
    assert st.sleeping_bodies == b.n - 1 - int((labels == labels[1]).sum())
    w.set_sleeping([1], True)
    sl = w.read_sleep()
    assert sl["sleeping"][1] == 1 and sl["island"][1] == 1
    with pytest.raises(ax.AxiomError) as e:
        w.set_sleeping([b.n + 5], False)
    assert e.value.code == 601  # OutOfRange
    w.set_sleeping([0], True)  # a static plane: left alone
    assert w.read_sleep()["sleeping"][0] == 0


def test_oracle_sleep_off_by_default(oracle):
    b = stacks()
    w = ax.PhysicsWorld(ax.default_config(oracle, time_step=DT), lib=oracle)
    assert w.config.allow_sleep == 0
    assert w.config.sleep_time_threshold == pytest.approx(0.5)
    assert w.config.sleep_linear_threshold == pytest.approx(0.01)
    w.add_bodies(b)
    for _ in range(80):
        st = w.step(DT)
    assert st.sleeping_bodies == 0 and st.island_count == 0 and st.active_bodies == b.n - 1
    sl = w.read_sleep()
    assert not sl["sleeping"].any() and (sl["island"] == 0xFFFFFFFF).all()
    with pytest.raises(ax.AxiomError) as e:
        w.set_sleeping([1], True)
    assert e.value.code == 600  # InvalidParameter
    with pytest.raises(ax.AxiomError):
        ax.PhysicsWorld(ax.default_config(oracle, allow_sleep=1, sleep_time_threshold=0.0), lib=oracle)


def test_oracle_body_that_may_not_sleep_keeps_its_island_awake(oracle):
    b = stacks()
    allow = np.ones(b.n, np.uint8)
    allow[1] = 0  # the first stack's bottom box
    b2 = ax.Bodies(**dict(b.arrays, allow_sleep=allow))
    w = world(oracle, b2)
    for _ in range(150):
        st = w.step(DT)
    sl = w.read_sleep()
    labels = stack_labels(b)
    mine = labels == labels[1]
    assert not sl["sleeping"][mine].any()
    assert sl["sleeping"][1:][~mine[1:]].all()
    assert st.sleeping_bodies == b.n - 1 - int(mine.sum())


def test_oracle_added_asleep_and_kinematic_mover_wakes(oracle):
    # a box added asleep in mid-air stays put; a moving kinematic box pushing into it
    # wakes it, after which it falls
    b = ax.Bodies(type=[ax.BODY_DYNAMIC, ax.BODY_KINEMATIC], shape=[ax.SHAPE_BOX, ax.SHAPE_BOX],
                  position=[(0.0, 5.0, 0.0), (-3.0, 5.0, 0.0)], shape_extents=[(H, H, H)] * 2,
                  linear_velocity=[(0.0, 0.0, 0.0), (2.0, 0.0, 0.0)], is_sleeping=np.array([1, 0], np.uint8))
    w = world(oracle, b)
    st = w.step(DT)
    assert st.sleeping_bodies == 1
    y0 = w.read_state()["position"][0, 1]
    assert y0 == np.float32(5.0)
    for k in range(120):
        st = w.step(DT)
        if st.sleeping_bodies == 0:
            break
    else:
        raise AssertionError("the kinematic box never woke the sleeper")
    assert st.manifold_count >= 1
    for _ in range(10):
        w.step(DT)
    assert w.read_state()["position"][0, 1] < 5.0 - 1e-3


# ------------------------------------------------------------ GPU vs oracle ----

def lockstep(lib, oracle, bodies, steps, before_step=None, **cfg):
    g, o = world(lib, bodies, **cfg), world(oracle, bodies, **cfg)
    oracle.oracle_set_threads(o.handle, 8)
    for k in range(steps):
        if before_step:
            before_step(k, g, o)
        sg, so = g.step(DT), o.step(DT)
        for f in ("pair_count", "manifold_count", "contact_point_count", "colour_count", "sleeping_bodies",
                  "active_bodies", "island_count", "dynamic_bodies"):
            assert getattr(sg, f) == getattr(so, f), (k, f, getattr(sg, f), getattr(so, f))
        a, b = g.read_state(), o.read_state()
        for key in a:
            assert np.array_equal(a[key], b[key]), (k, key)
        la, lb = g.read_sleep(), o.read_sleep()
        for key in la:
            assert np.array_equal(la[key], lb[key]), (k, key)
    return g, o


@pytest.mark.gpu
def test_gpu_sleep_and_wake_bit_exact(gpu_lib, oracle):
    b = stacks()
    dropped = {}

    def drop(k, g, o):
        if k == 90:  # everything sleeps by now
            assert g.read_sleep()["sleeping"][1:].all()
            sid_g, ids = drop_on_tallest(g, b)
            sid_o, _ = drop_on_tallest(o, b)
            assert sid_g == sid_o
            dropped["ids"] = ids

    g, o = lockstep(gpu_lib, oracle, b, 220, drop)
    assert "ids" in dropped


@pytest.mark.gpu
def test_gpu_set_sleeping_and_mover_bit_exact(gpu_lib, oracle):
    base = stacks(3, 3)
    allow = np.ones(base.n, np.uint8)
    allow[-1] = 0  # the last box never sleeps, nor does its island
    base = ax.Bodies(**dict(base.arrays, allow_sleep=allow))
    # a kinematic box sliding into the first stack, and a box added asleep in mid-air
    extra = ax.Bodies(type=[ax.BODY_KINEMATIC, ax.BODY_DYNAMIC], shape=[ax.SHAPE_BOX, ax.SHAPE_BOX],
                      position=[(-6.0, H, 0.0), (0.0, 6.0, 9.0)], shape_extents=[(H, H, H)] * 2,
                      linear_velocity=[(0.05, 0.0, 0.0), (0.0, 0.0, 0.0)],
                      is_sleeping=np.array([0, 1], np.uint8))
    b = concat(base, extra)

    def poke(k, g, o):
        if k == 100:
            for w in (g, o):
                w.set_sleeping([2, 3], False)
        if k == 130:
            for w in (g, o):
                w.set_sleeping([1], True)

    lockstep(gpu_lib, oracle, b, 200, poke)


@pytest.mark.gpu
def test_gpu_sphere_lattice_islands_bit_exact(gpu_lib, oracle):
    # a collapsing sphere lattice: many islands merging and splitting, loose thresholds so
    # that some islands sleep and wake again
    sc = ax.Scene.sphere_lattice(seed=3, dims=(8, 3, 8), spacing=0.49, radius=0.25, jitter=0.002, lib=gpu_lib)
    lockstep(gpu_lib, oracle, sc.bodies, 150, sleep_linear_threshold=0.3, sleep_angular_threshold=1.0,
             sleep_time_threshold=0.1)
