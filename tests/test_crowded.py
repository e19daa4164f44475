"""Bodies with more manifolds than the colouring can separate.

A contact graph is coloured with at most 64 colours, so a dynamic body touching more than
a few dozen others cannot have all its manifolds in distinct colours of a two-sided
greedy colouring.  A manifold at a dynamic body with more than 32 manifolds is therefore
"crowded": it takes no colour (64) and is solved in one serial batch after the colours, in
descending priority; every other manifold always finds a colour.  The tests drop a
dynamic box onto 100 spheres and a heavy plate onto 400 (the box's and plate's manifolds
are crowded), check the step succeeds and holds the bodies up, and that the GPU matches
the oracle bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax

DT = 1.0 / 120.0


def plate_on_spheres(side=10, r=0.25, mass=500.0):
    """side x side spheres on the ground in a square grid, a dynamic plate resting on all."""
    he = (0.3 * side, 0.25, 0.3 * side)
    k = np.arange(side)
    x, z = np.meshgrid((k - (side - 1) / 2) * 0.55, (k - (side - 1) / 2) * 0.55, indexing="ij")
    n = side * side
    pos = np.column_stack([x.ravel(), np.full(n, r), z.ravel()])
    box = [0.0, 2 * r + he[1] - 0.002, 0.0]
    return ax.Bodies(type=np.r_[np.ones(n + 1), 0].astype(np.uint32),
                     shape=np.r_[np.full(n, ax.SHAPE_SPHERE), ax.SHAPE_BOX, ax.SHAPE_PLANE].astype(np.uint32),
                     position=np.vstack([pos, [box], [[0.0, 0.0, 0.0]]]).astype(np.float32),
                     shape_extents=np.vstack([np.tile([r, 0, 0], (n, 1)), [he], [[0, 0, 0]]]).astype(np.float32),
                     mass=np.r_[np.full(n, 60.0), mass, 0.0].astype(np.float32),
                     restitution=np.zeros(n + 2, np.float32))


@pytest.mark.parametrize("side", [10, 20])
def test_oracle_crowded_box_is_solved(oracle, side):
    b = plate_on_spheres(side)
    w = ax.PhysicsWorld(ax.default_config(oracle, time_step=DT, velocity_iterations=10), lib=oracle)
    w.add_bodies(b)
    box = side * side
    for _ in range(30):
        st = w.step(DT)
        assert st.status == 0
    c = w.read_contacts()
    at_box = (c["body_a"] == box) | (c["body_b"] == box)
    assert at_box.sum() == side * side  # one point per sphere under the plate
    assert (c["colour"][at_box] == 64).all()  # crowded
    y = w.read_state()["position"][box, 1]
    assert y > 2 * 0.25 + 0.25 - 0.03  # held up by the spheres (not sunk through)


@pytest.mark.gpu
@pytest.mark.parametrize("side", [10, 20])
def test_gpu_crowded_box_bit_exact(gpu_lib, oracle, side):
    from test_gpu_parity import compare_step, make_worlds

    g, o = make_worlds(gpu_lib, oracle, plate_on_spheres(side), time_step=DT, velocity_iterations=10)
    for k in range(30):
        sg, so = g.step(DT), o.step(DT)
        assert (sg.status, sg.colour_count, sg.iterations, sg.residual) == \
            (so.status, so.colour_count, so.iterations, so.residual), k
        compare_step(g, o, k)
    for mode in (dict(temporal_colouring=1), dict(residual_tolerance=1e-4, max_iterations=400)):
        g, o = make_worlds(gpu_lib, oracle, plate_on_spheres(side), time_step=DT, **mode)
        for k in range(20):
            sg, so = g.step(DT, check=False), o.step(DT, check=False)
            assert (sg.iterations, sg.residual) == (so.iterations, so.residual), (mode, k)
            compare_step(g, o, k)
