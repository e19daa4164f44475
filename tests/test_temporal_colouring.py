"""Temporally coherent colouring (axiom_world_config.temporal_colouring).

A manifold that existed in the previous step keeps its colour unless a higher-priority
manifold that also existed keeps the same colour at a shared dynamic body; the rest are
coloured greedily in descending priority around the kept colours.  The CPU tests check,
on the oracle, that the colouring stays proper (no two manifolds of one colour share a
dynamic body), that a settled pile keeps its colours and recolours only its new contacts
(the colouring's dependency depth falls to the new contacts'), and that a snapshot carries
the colours so that a resumed world continues bit for bit.  The GPU tests check the CUDA
library against the oracle with the option on: pairs, colours, contacts, impulses and
state bit-exact, on a sphere drop (contacts appear every step), a walled pile, mixed
shapes and a sleeping scene, plus a cross-implementation snapshot resume.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import axiom_gb300 as ax
import bench
from test_gpu_parity import compare_step

DT = 1.0 / 120.0


def proper(contacts, types):
    """No dynamic body has two manifolds of the same colour."""
    c0 = contacts[contacts["point_index"] == 0]
    keys = []
    for side in ("body_a", "body_b"):
        dyn = types[c0[side]] == ax.BODY_DYNAMIC
        keys.append(np.stack([c0[side][dyn], c0["colour"][dyn]], 1))
    keys = np.concatenate(keys)
    return len(np.unique(keys, axis=0)) == len(keys)


def colours_by_pair(contacts):
    c0 = contacts[contacts["point_index"] == 0]
    return {(int(a), int(b)): int(c) for a, b, c in zip(c0["body_a"], c0["body_b"], c0["colour"])}


def test_oracle_temporal_colouring_proper_and_coherent(oracle, lib):
    sc = bench.pile_scene(lib, (16, 12, 16))
    types = sc.bodies.arrays["type"]
    w = ax.PhysicsWorld(bench.pile_config(oracle, temporal_colouring=1), lib=oracle)
    w.add_bodies(sc.bodies)
    st = w.step(bench.DT)
    first_rounds = st.colour_rounds
    prev = colours_by_pair(w.read_contacts())
    assert proper(w.read_contacts(), types)
    for _ in range(6):
        st = w.step(bench.DT)
        c = w.read_contacts()
        assert proper(c, types)
        now = colours_by_pair(c)
        kept = sum(1 for k, v in now.items() if prev.get(k) == v)
        # the pile is settled: almost every manifold persists with its colour
        assert kept >= 0.97 * len(now)
        prev = now
    assert first_rounds > 10 and st.colour_rounds <= 2


def test_oracle_temporal_colouring_matches_greedy_on_first_step(oracle, lib):
    """With no previous colours the temporal mode is the greedy colouring."""
    sc = ax.Scene.sphere_drop(seed=1, count=400, size=(8.0, 30.0, 8.0), lib=lib)
    a = ax.PhysicsWorld(ax.default_config(oracle, time_step=DT), lib=oracle)
    b = ax.PhysicsWorld(ax.default_config(oracle, time_step=DT, temporal_colouring=1), lib=oracle)
    a.add_bodies(sc.bodies)
    b.add_bodies(sc.bodies)
    for _ in range(80):  # until the spheres have landed and touch
        sa, sb = a.step(DT), b.step(DT)
        if sa.manifold_count:
            break
    assert sa.manifold_count > 0
    assert np.array_equal(ax.canonical_contacts(a.read_contacts()), ax.canonical_contacts(b.read_contacts()))


def test_oracle_temporal_snapshot_resumes_bit_exact(oracle, lib):
    sc = ax.Scene.mixed(seed=11, count=500, size=(10.0, 14.0, 10.0), lib=lib)
    w = ax.PhysicsWorld(ax.default_config(oracle, time_step=DT, temporal_colouring=1), lib=oracle)
    w.add_bodies(sc.bodies)
    for _ in range(40):
        w.step(DT, check=False)
    snap = w.save_snapshot()
    h, _, contacts, _ = ax.parse_snapshot(snap)
    assert h.version == 3 and h.config.temporal_colouring == 1
    tags = contacts["point"] >> 8
    assert (tags[(contacts["point"] & 0xFF) == 0] > 0).all() and (tags[(contacts["point"] & 0xFF) > 0] == 0).all()
    r = ax.PhysicsWorld(ax.default_config(oracle, time_step=DT), lib=oracle)
    r.load_snapshot(snap)
    assert r.save_snapshot() == snap
    for _ in range(20):
        sw, sr = w.step(DT, check=False), r.step(DT, check=False)
        assert sw.colour_rounds == sr.colour_rounds
    a, b = w.read_state(), r.read_state()
    assert all(np.array_equal(a[k], b[k]) for k in a)


def test_batch_rejects_temporal_colouring(lib):
    with pytest.raises(ax.AxiomError) as e:
        ax.Batch(ax.default_config(lib, temporal_colouring=1), lib=lib)
    assert e.value.code in (ax.ERR_INVALID_PARAMETER, 505)  # 505 where no GPU is present


def conflicting_snapshot(blob: bytes, every: int) -> bytes:
    """The snapshot with the previous colour of every `every`-th manifold (point-0 entry)
    set to colour 0, so that manifolds at one dynamic body share previous colours."""
    h, bodies, contacts, _ = ax.parse_snapshot(blob)
    out = bytearray(blob)
    off = ctypes.sizeof(ax.SnapshotHeader) + ax.SNAPSHOT_BODY_DTYPE.itemsize * h.body_count
    c = np.frombuffer(out, ax.SNAPSHOT_CONTACT_DTYPE, h.contact_count, off)
    c = c.copy()
    first = np.flatnonzero((c["point"] & 0xFF) == 0)[::every]
    c["point"][first] = (c["point"][first] & ~np.uint32(0xFF00)) | np.uint32(1 << 8)
    out[off:off + c.nbytes] = c.tobytes()
    return bytes(out)


def test_oracle_temporal_conflicting_previous_colours(oracle, lib):
    """Previous colours that clash at a body (from an edited snapshot) are resolved: the
    lower-priority manifold is recoloured and the colouring stays proper."""
    sc = bench.pile_scene(lib, (12, 8, 12))
    types = sc.bodies.arrays["type"]
    w = ax.PhysicsWorld(bench.pile_config(oracle, temporal_colouring=1), lib=oracle)
    w.add_bodies(sc.bodies)
    for _ in range(3):
        w.step(bench.DT)
    for every in (1, 7):
        w.load_snapshot(conflicting_snapshot(w.save_snapshot(), every))
        st = w.step(bench.DT)
        assert proper(w.read_contacts(), types)
        assert st.colour_rounds > 2  # the dropped manifolds were recoloured through the chains


# ------------------------------------------------------------------------ GPU ----

def _run_pair(gpu_lib, oracle, bodies, steps, check=True, **cfg):
    from test_gpu_parity import make_worlds

    g, o = make_worlds(gpu_lib, oracle, bodies, temporal_colouring=1, **cfg)
    rounds = []
    for k in range(steps):
        sg, so = g.step(cfg.get("time_step", DT), check=check), o.step(cfg.get("time_step", DT), check=check)
        assert (sg.pair_count, sg.manifold_count, sg.colour_count, sg.colour_rounds, sg.iterations) == \
            (so.pair_count, so.manifold_count, so.colour_count, so.colour_rounds, so.iterations), k
        compare_step(g, o, k)
        rounds.append(sg.colour_rounds)
    return g, o, rounds


@pytest.mark.gpu
def test_gpu_temporal_sphere_drop_bit_exact(gpu_lib, oracle):
    sc = ax.Scene.sphere_drop(seed=1, lib=gpu_lib)
    _run_pair(gpu_lib, oracle, sc.bodies, 120, time_step=DT, velocity_iterations=10)


@pytest.mark.gpu
def test_gpu_temporal_pile_bit_exact(gpu_lib, oracle):
    sc = bench.pile_scene(gpu_lib, (24, 16, 24))
    _, _, rounds = _run_pair(gpu_lib, oracle, sc.bodies, 20, time_step=bench.DT, velocity_iterations=10,
                             linear_slop=bench.SLOP)
    assert rounds[0] > 10 and max(rounds[1:]) <= 2  # only new contacts are recoloured


@pytest.mark.gpu
def test_gpu_temporal_mixed_shapes_bit_exact(gpu_lib, oracle):
    sc = ax.Scene.mixed(seed=2, count=3000, size=(20.0, 30.0, 20.0), lib=gpu_lib)
    _run_pair(gpu_lib, oracle, sc.bodies, 40, check=False, time_step=DT, velocity_iterations=20)


@pytest.mark.gpu
def test_gpu_temporal_sleeping_bit_exact(gpu_lib, oracle):
    sc = ax.Scene.towers(seed=5, count=8, lib=gpu_lib)
    _run_pair(gpu_lib, oracle, sc.bodies, 60, check=False, time_step=1 / 60, velocity_iterations=10,
              allow_sleep=1, sleep_linear_threshold=0.05, sleep_angular_threshold=0.1, sleep_time_threshold=0.2)


@pytest.mark.gpu
def test_gpu_temporal_conflicting_previous_colours_bit_exact(gpu_lib, oracle):
    """Clashing previous colours take the second linking pass on the GPU (conflict found,
    manifolds dropped, links redone); the result equals the oracle's bit for bit.  The
    (12, 8, 12) pile is a small world, coloured and solved by the single-CTA kernels; the
    (24, 16, 24) pile takes the multi-launch colouring and colour passes."""
    for dims in ((12, 8, 12), (24, 16, 24)):
        for every in (1, 5):
            _conflicting_resume(gpu_lib, oracle, dims, every)


def _conflicting_resume(gpu_lib, oracle, dims, every):
    from test_gpu_parity import make_worlds

    sc = bench.pile_scene(gpu_lib, dims)
    cfg = dict(time_step=bench.DT, velocity_iterations=10, linear_slop=bench.SLOP, temporal_colouring=1)
    o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    o.add_bodies(sc.bodies)
    for _ in range(3):
        o.step(bench.DT)
    blob = conflicting_snapshot(o.save_snapshot(), every)
    g, o2 = make_worlds(gpu_lib, oracle, sc.bodies, **cfg)
    g.load_snapshot(blob)
    o2.load_snapshot(blob)
    for k in range(3):
        sg, so = g.step(bench.DT), o2.step(bench.DT)
        assert (sg.manifold_count, sg.colour_count, sg.colour_rounds, sg.iterations) == \
            (so.manifold_count, so.colour_count, so.colour_rounds, so.iterations), (dims, every, k)
        compare_step(g, o2, k)
    assert proper(g.read_contacts(), sc.bodies.arrays["type"])


@pytest.mark.gpu
def test_gpu_temporal_snapshot_cross_resume(gpu_lib, oracle):
    sc = ax.Scene.sphere_drop(seed=3, count=600, size=(10.0, 30.0, 10.0), lib=gpu_lib)
    g, o, _ = _run_pair(gpu_lib, oracle, sc.bodies, 90, time_step=DT, velocity_iterations=10)
    sg, so = g.save_snapshot(), o.save_snapshot()
    assert sg == so
    # each resumes the other's snapshot and both keep stepping identically
    g2 = ax.PhysicsWorld(ax.default_config(gpu_lib, time_step=DT), lib=gpu_lib)
    o2 = ax.PhysicsWorld(ax.default_config(oracle, time_step=DT), lib=oracle)
    g2.load_snapshot(so)
    o2.load_snapshot(sg)
    for k in range(20):
        a, b = g2.step(DT), o2.step(DT)
        assert a.colour_rounds == b.colour_rounds
        compare_step(g2, o2, k)
