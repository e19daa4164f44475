"""Mid-size worlds solve in one thread-block-cluster launch.

A world above the single-CTA bounds (more than 4,096 manifolds or bodies) and with at most
32,768 manifolds (65,536 when every manifold has one point), or within them with more than
1,024 manifolds some of which have several points, runs its warm start, every sweep and the convergence test in one launch of
one cluster: colours follow each other at cluster barriers, the crowded batch is sorted in
global scratch and solved by one thread after the colours, and the sweep maxima meet in
rotating counter pairs.  Each case checks that the step took that path (one solve launch
per step, no separate warm-start launches) and matches the CPU oracle bit for bit:

  a 3,200-sphere lattice with fixed sweeps, and in tolerance mode (same sweep counts and
  residuals);
  box towers in tolerance mode (four-point manifolds), and 48 towers (a world within the
  single-CTA bounds that takes the cluster for its four-point manifolds);
  a plate on 4,900 spheres (more than 4,096 crowded manifolds: the sort's scratch is larger
  than any shared-memory buffer of the single-CTA solve);
  spheres apart on a dynamic plate (every manifold is crowded: sweeps with no colour).
"""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax
from test_crowded import plate_on_spheres
from test_gpu_parity import compare_step, make_worlds

pytestmark = pytest.mark.gpu

DT = 1.0 / 120.0


def spheres_on_plate(side=70, r=0.25, gap=0.1, plate_mass=5000.0):
    """A dynamic plate on the ground, side x side spheres resting on it, apart from each
    other: every manifold is at the plate, which has more than 32 of them."""
    pitch = 2 * r + gap
    he = (0.5 * side * pitch + 0.5, 0.25, 0.5 * side * pitch + 0.5)
    k = np.arange(side)
    x, z = np.meshgrid((k - (side - 1) / 2) * pitch, (k - (side - 1) / 2) * pitch, indexing="ij")
    n = side * side
    plate_y = he[1] - 0.002
    pos = np.column_stack([x.ravel(), np.full(n, plate_y + he[1] + r - 0.002), z.ravel()])
    return ax.Bodies(type=np.r_[np.ones(n + 1), 0].astype(np.uint32),
                     shape=np.r_[np.full(n, ax.SHAPE_SPHERE), ax.SHAPE_BOX, ax.SHAPE_PLANE].astype(np.uint32),
                     position=np.vstack([pos, [[0.0, plate_y, 0.0]], [[0.0, 0.0, 0.0]]]).astype(np.float32),
                     shape_extents=np.vstack([np.tile([r, 0, 0], (n, 1)), [he], [[0, 0, 0]]]).astype(np.float32),
                     mass=np.r_[np.full(n, 1.0), plate_mass, 0.0].astype(np.float32),
                     restitution=np.zeros(n + 2, np.float32))


def run_compared(g, o, steps, dt=DT):
    g.reset_profile()
    for k in range(steps):
        sg, so = g.step(dt, check=False), o.step(dt, check=False)
        assert (sg.status, sg.colour_count, sg.iterations, sg.residual) == \
            (so.status, so.colour_count, so.iterations, so.residual), k
        assert 4096 < sg.manifold_count <= 65536 or sg.total_bodies > 4096, k
        compare_step(g, o, k)
    prof = g.read_profile()
    assert prof["pgs_colour"]["launches"] == steps  # one cluster launch per step
    assert prof["warm_start_apply"]["launches"] == 0
    return sg


def test_cluster_lattice_fixed_and_tolerance(gpu_lib, oracle):
    sc = ax.Scene.sphere_lattice(seed=5, dims=(20, 8, 20), lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=DT, velocity_iterations=10)
    st = run_compared(g, o, 8)
    assert 4096 < st.manifold_count <= 32768 and st.colour_count > 1
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=DT, residual_tolerance=1e-4, max_iterations=500)
    st = run_compared(g, o, 4)
    assert st.iterations > 10


def test_cluster_towers_tolerance(gpu_lib, oracle):
    sc = ax.Scene.towers(seed=5, count=160, lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=1 / 60, residual_tolerance=1e-4, max_iterations=200)
    run_compared(g, o, 6, dt=1 / 60)
    assert (g.read_contacts()["point_index"] == 3).any()


def test_cluster_small_multipoint(gpu_lib, oracle):
    sc = ax.Scene.towers(seed=5, count=48, lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=1 / 60, velocity_iterations=20)
    g.reset_profile()
    for k in range(14):
        sg, so = g.step(1 / 60, check=False), o.step(1 / 60, check=False)
        assert (sg.status, sg.colour_count, sg.iterations, sg.residual) == \
            (so.status, so.colour_count, so.iterations, so.residual), k
        if k >= 10:  # settled into contact: within the single-CTA bounds, above 1,024, multi-point
            assert 1024 < sg.manifold_count <= 4096 and sg.contact_point_count > sg.manifold_count, k
        compare_step(g, o, k)
    prof = g.read_profile()
    assert prof["pgs_colour"]["launches"] == 14 and prof["warm_start_apply"]["launches"] == 0


def test_cluster_single_point_above_multipoint_limit(gpu_lib, oracle):
    sc = ax.Scene.sphere_lattice(seed=5, dims=(48, 8, 48), lib=gpu_lib)
    g, o = make_worlds(gpu_lib, oracle, sc.bodies, time_step=DT, velocity_iterations=10)
    st = run_compared(g, o, 3)
    assert 32768 < st.manifold_count <= 65536 and st.contact_point_count == st.manifold_count


def test_cluster_many_crowded(gpu_lib, oracle):
    g, o = make_worlds(gpu_lib, oracle, plate_on_spheres(70), time_step=DT, velocity_iterations=10)
    st = run_compared(g, o, 3)
    c = g.read_contacts()
    assert (c["colour"] == 64).sum() > 4096 and st.colour_count >= 1


def test_cluster_all_crowded(gpu_lib, oracle):
    g, o = make_worlds(gpu_lib, oracle, spheres_on_plate(70), time_step=DT, velocity_iterations=10)
    st = run_compared(g, o, 3)
    c = g.read_contacts()
    assert len(c) > 4096 and (c["colour"] == 64).all() and st.colour_count == 0
