"""GPU step vs the CPU oracle on identical seeded inputs, through the C ABI.

Bars (from the step's contract): broadphase pair sets and colour assignments bit-exact
after canonical sorting; contact normals, points and depths within 1e-5 relative;
impulses within 1e-4 relative under the same colour order; trajectories within 1e-3 m
over 120 steps at dt = 1/120 s.  Both sides evaluate the same fp32 expressions without
fused multiply-add, so the tests also assert the stronger bit-exact equality.
"""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax

pytestmark = pytest.mark.gpu

REL_CONTACT = 1e-5
REL_IMPULSE = 1e-4
TRAJ_M = 1e-3


def make_worlds(lib, oracle, bodies, threads=8, **cfg):
    g = ax.PhysicsWorld(ax.default_config(lib, **cfg), lib=lib)
    o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    oracle.oracle_set_threads(o.handle, threads)
    g.add_bodies(bodies)
    o.add_bodies(bodies)
    return g, o


def rel_close(a, b, rel, floor=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.all(np.abs(a - b) <= rel * np.maximum(np.maximum(np.abs(a), np.abs(b)), floor))


def compare_step(g, o, step_no, exact=True):
    pg = ax.canonical_pairs(g.read_pairs())
    po = ax.canonical_pairs(o.read_pairs())
    assert np.array_equal(pg, po), f"step {step_no}: pair sets differ ({len(pg)} vs {len(po)})"
    cg = ax.canonical_contacts(g.read_contacts())
    co = ax.canonical_contacts(o.read_contacts())
    assert len(cg) == len(co), f"step {step_no}: contact counts {len(cg)} vs {len(co)}"
    for f in ("body_a", "body_b", "point_index", "colour"):
        assert np.array_equal(cg[f], co[f]), f"step {step_no}: {f} differs"
    for f in ("position", "normal", "penetration_depth"):
        assert rel_close(cg[f], co[f], REL_CONTACT), f"step {step_no}: {f} beyond 1e-5 relative"
    assert rel_close(cg["impulse"], co["impulse"], REL_IMPULSE), f"step {step_no}: impulses"
    sg, so = g.read_state(), o.read_state()
    dmax = float(np.abs(sg["position"] - so["position"]).max()) if len(sg["position"]) else 0.0
    assert dmax <= TRAJ_M, f"step {step_no}: trajectory drift {dmax}"
    if exact:
        for f in ("position", "normal", "penetration_depth", "impulse"):
            assert np.array_equal(cg[f], co[f]), f"step {step_no}: {f} not bit-exact"
        for k in sg:
            assert np.array_equal(sg[k], so[k]), f"step {step_no}: state {k} not bit-exact"
    return len(pg), len(cg)


def test_sphere_drop_1k_120_steps(gpu_lib, oracle):
    """1,000 spheres (r 0.5, rho 1000) dropped on a plane: dt 1/120, 10 PGS sweeps."""
    sc = ax.Scene.sphere_drop(seed=1, lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=1 / 120, velocity_iterations=10)
    contacts = 0
    for k in range(120):
        sg = g.step(1 / 120)
        so = o.step(1 / 120)
        assert sg.pair_count == so.pair_count and sg.manifold_count == so.manifold_count
        assert sg.colour_count == so.colour_count and sg.iterations == so.iterations
        assert sg.residual == so.residual
        _, c = compare_step(g, o, k)
        contacts += c
    assert contacts > 1000  # the spheres do land and pile


def test_lattice_small_bit_exact(gpu_lib, oracle):
    """A 24x12x24 jittered lattice: ~13 AABB pairs and ~3 contacts per sphere."""
    sc = ax.Scene.sphere_lattice(seed=3, dims=(24, 12, 24), lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=1 / 120, velocity_iterations=10)
    for k in range(8):
        sg = g.step(1 / 120)
        so = o.step(1 / 120)
        p, c = compare_step(g, o, k)
        assert p > 12 * 24 * 12 * 24 * 0.9 and c > 2 * 24 * 12 * 24
        # parallel colouring rounds = longest chain of higher-priority neighbours
        assert sg.colour_rounds == so.colour_rounds and sg.colour_rounds > 1


def test_per_iteration_impulses(gpu_lib, oracle):
    """Impulses after 1..10 sweeps agree (same colour order on both sides)."""
    sc = ax.Scene.sphere_lattice(seed=11, dims=(12, 6, 12), lib=gpu_lib)
    for iters in (1, 2, 5, 10):
        g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=1 / 120, velocity_iterations=iters)
        for k in range(3):
            g.step(1 / 120)
            o.step(1 / 120)
        compare_step(g, o, iters)


def test_tolerance_mode_matches(gpu_lib, oracle):
    """Residual-threshold mode: same sweep count and residual on both sides."""
    sc = ax.Scene.sphere_lattice(seed=5, dims=(10, 10, 10), lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=1 / 120, residual_tolerance=1e-4,
                       max_iterations=500)
    for k in range(4):
        sg = g.step(1 / 120, check=False)
        so = o.step(1 / 120, check=False)
        assert sg.status == so.status
        assert sg.iterations == so.iterations and sg.residual == so.residual
        compare_step(g, o, k)


def test_colouring_is_valid(gpu_lib):
    sc = ax.Scene.sphere_lattice(seed=3, dims=(20, 10, 20), lib=gpu_lib)
    g = ax.PhysicsWorld(ax.default_config(gpu_lib, time_step=1 / 120), lib=gpu_lib)
    g.add_bodies(sc.bodies)
    g.step(1 / 120)
    c = g.read_contacts()
    dyn = sc.bodies.arrays["type"] == ax.BODY_DYNAMIC
    for col in np.unique(c["colour"]):
        sel = c[c["colour"] == col]
        man = np.unique(np.stack([sel["body_a"], sel["body_b"]], 1), axis=0)
        ids = man.reshape(-1)
        ids = ids[dyn[ids]]
        assert len(ids) == len(np.unique(ids)), f"colour {col} reuses a dynamic body"


def test_gpu_runs_are_deterministic(gpu_lib):
    sc = ax.Scene.sphere_lattice(seed=9, dims=(16, 8, 16), lib=gpu_lib)
    states = []
    for _ in range(2):
        g = ax.PhysicsWorld(ax.default_config(gpu_lib, time_step=1 / 120, velocity_iterations=10),
                            lib=gpu_lib)
        g.add_bodies(sc.bodies)
        for _ in range(10):
            g.step(1 / 120)
        states.append(g.read_state())
    for k in states[0]:
        assert states[0][k].tobytes() == states[1][k].tobytes()


def test_empty_world_and_no_contacts(gpu_lib):
    g = ax.PhysicsWorld(ax.default_config(gpu_lib), lib=gpu_lib)
    st = g.step()
    assert st.total_bodies == 0 and st.pair_count == 0
    b = ax.Bodies(type=[1, 1], shape=[0, 0], position=[[0, 10, 0], [5, 10, 0]],
                  shape_extents=[[0.5, 0, 0], [0.5, 0, 0]])
    g.add_bodies(b)
    st = g.step()
    assert st.pair_count == 0 and st.manifold_count == 0
    s = g.read_state()
    assert s["linear_velocity"][0, 1] < 0


def test_pair_capacity_overflow_grows(gpu_lib, oracle):
    """A deliberately tiny pair capacity makes the step grow its buffers and redo the stage."""
    sc = ax.Scene.sphere_lattice(seed=3, dims=(12, 6, 12), lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=1 / 120, pair_capacity=16,
                       contact_capacity=16)
    g.step(1 / 120)
    o.step(1 / 120)
    compare_step(g, o, 0)


def test_full_lattice_pairs_match_oracle(gpu_lib, oracle):
    """The 1,048,576-sphere pile: one step, pair set bit-exact against the oracle."""
    sc = ax.Scene.sphere_lattice(seed=3, lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, threads=16, time_step=1 / 120,
                       velocity_iterations=10)
    sg = g.step(1 / 120)
    so = o.step(1 / 120)
    assert sg.pair_count == so.pair_count > 12_000_000
    assert np.array_equal(ax.canonical_pairs(g.read_pairs()), ax.canonical_pairs(o.read_pairs()))
    assert sg.manifold_count == so.manifold_count and sg.colour_count == so.colour_count
    sgs, sos = g.read_state(), o.read_state()
    for k in sgs:
        assert np.array_equal(sgs[k], sos[k]), k


def shape_mix(contacts, shapes):
    """Counts of manifold shape combinations, for coverage assertions."""
    a = shapes[contacts["body_a"]]
    b = shapes[contacts["body_b"]]
    return {(int(x), int(y)) for x, y in zip(a, b)}


def test_mixed_shapes_bit_exact(gpu_lib, oracle):
    """Spheres, boxes and capsules (40/40/20 %) dropped into a dense box: every analytic
    pair type plus GJK/EPA box-box and box-capsule, compared for 60 steps."""
    sc = ax.Scene.mixed(seed=2, count=4000, size=(24.0, 30.0, 24.0), lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=1 / 120, velocity_iterations=20)
    shapes = sc.bodies.arrays["shape"]
    seen = set()
    gjk_failures = 0
    for k in range(60):
        sg = g.step(1 / 120)
        so = o.step(1 / 120)
        compare_step(g, o, k)
        assert sg.colour_rounds == so.colour_rounds
        # GJK / EPA convergence failures are reported alike (count and status)
        assert (sg.gjk_failures, sg.epa_failures, sg.status) == (so.gjk_failures, so.epa_failures, so.status), k
        gjk_failures += sg.gjk_failures
        seen |= shape_mix(g.read_contacts(), shapes)
    assert gjk_failures > 0  # this scene meets GJK pairs that run out of iterations
    B, S, C, P = ax.SHAPE_BOX, ax.SHAPE_SPHERE, ax.SHAPE_CAPSULE, ax.SHAPE_PLANE
    canon = {tuple(sorted(p)) for p in seen}
    for want in [(S, S), (S, B), (S, C), (B, B), (B, C), (C, C)]:
        assert tuple(sorted(want)) in canon, f"no {want} contact exercised"
    assert any(P in p for p in seen)


def test_towers_bit_exact(gpu_lib, oracle):
    """Box pyramids and towers (unit boxes, +-2 % jitter, friction 0.6): multi-point
    box-box and box-plane manifolds under the tolerance-mode solver."""
    sc = ax.Scene.towers(seed=5, count=12, lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=1 / 60, residual_tolerance=1e-4,
                       max_iterations=60)
    for k in range(30):
        sg = g.step(1 / 60, check=False)
        so = o.step(1 / 60, check=False)
        assert sg.iterations == so.iterations and sg.residual == so.residual
        compare_step(g, o, k)
    c = g.read_contacts()
    assert (c["point_index"] == 3).any()  # 4-point manifolds present
