"""Static triangle meshes (gui::ShapeType::Mesh, include/axiom/gui/body_inspector.hpp:25).

A mesh is added as one static body per triangle, each a flat three-point hull about its
centroid (shape AXIOM_SHAPE_MESH), so the broadphase, GJK / EPA, the supporting-feature
clipper, colouring, warm start, sleeping and snapshots treat triangles like any static body.
The tests check resting heights on a tessellated floor, motion down a ramp, the entry
point's validation, snapshot round trips and bit-exact GPU-vs-oracle stepping over terrain.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import axiom_gb300 as ax

DT = 1.0 / 120.0


def grid_mesh(nx=12, nz=12, cell=1.0, height=None):
    """A tessellated surface over [0, nx*cell] x [0, nz*cell]; height(x, z) -> y (flat if None)."""
    xs = np.arange(nx + 1) * cell
    zs = np.arange(nz + 1) * cell
    X, Z = np.meshgrid(xs, zs, indexing="ij")
    Y = np.zeros_like(X) if height is None else height(X, Z)
    verts = np.column_stack([X.ravel(), Y.ravel(), Z.ravel()]).astype(np.float32)
    idx = lambda i, k: i * (nz + 1) + k
    tris = []
    for i in range(nx):
        for k in range(nz):
            a, b, c, d = idx(i, k), idx(i + 1, k), idx(i + 1, k + 1), idx(i, k + 1)
            tris += [(a, c, b), (a, d, c)]  # counter-clockwise seen from +y
    return verts, np.array(tris, np.uint32)


def world(lib, **cfg):
    c = dict(time_step=DT, velocity_iterations=10)
    c.update(cfg)
    return ax.PhysicsWorld(ax.default_config(lib, **c), lib=lib)


def test_mesh_bodies_and_validation(oracle):
    w = world(oracle)
    v, t = grid_mesh(2, 2)
    first = w.add_triangle_mesh(v, t, friction=0.7)
    assert first == 0 and w.body_count() == len(t) == 8
    _, bodies, _, hulls = ax.parse_snapshot(w.save_snapshot())
    assert (bodies["shape"] == ax.SHAPE_MESH).all() and (bodies["type"] == ax.BODY_STATIC).all()
    assert np.allclose(bodies["friction"], 0.7)
    assert len(hulls) == 8 and all(h.shape == (3, 3) for h in hulls)
    # each triangle's points sum to ~0 about its centroid
    assert max(np.abs(h.sum(axis=0)).max() for h in hulls) < 1e-5
    with pytest.raises(ax.AxiomError) as e:
        w.add_triangle_mesh(v, [(0, 1, 99)])
    assert e.value.code == 601
    with pytest.raises(ax.AxiomError) as e:
        w.add_triangle_mesh(v, [(0, 1, 1)])  # no area
    assert e.value.code == 300
    with pytest.raises(ax.AxiomError):  # a mesh triangle may not be dynamic
        w.add_bodies(ax.Bodies(type=[1], shape=[ax.SHAPE_MESH], position=[(0, 0, 0)], shape_extents=[(0, 0, 0)],
                               convex_hull=[0]))


@pytest.mark.parametrize("shape, ext, rest_y", [
    (ax.SHAPE_SPHERE, (0.3, 0.0, 0.0), 0.3),
    (ax.SHAPE_BOX, (0.4, 0.25, 0.35), 0.25),
    (ax.SHAPE_CYLINDER, (0.3, 0.2, 0.0), 0.2),
])
def test_bodies_rest_on_mesh_floor(oracle, shape, ext, rest_y):
    w = world(oracle)
    v, t = grid_mesh()
    w.add_triangle_mesh(v, t, friction=0.6, restitution=0.0)
    first = w.add_bodies(ax.Bodies(type=[1], shape=[shape], position=[(5.3, 1.5, 6.7)], shape_extents=[ext],
                                   restitution=[0.0], friction=[0.6]))
    for _ in range(480):
        st = w.step(DT)
    s = w.read_state()
    assert abs(s["position"][first, 1] - rest_y) < 8e-3
    assert np.linalg.norm(s["linear_velocity"][first]) < 1e-2
    assert st.manifold_count >= 1


def test_sphere_rolls_down_mesh_ramp(oracle):
    slope = math.tan(math.radians(20.0))
    v, t = grid_mesh(16, 4, cell=1.0, height=lambda x, z: -slope * x)
    w = world(oracle)
    w.add_triangle_mesh(v, t, friction=0.6, restitution=0.0)
    first = w.add_bodies(ax.Bodies(type=[1], shape=[ax.SHAPE_SPHERE], position=[(1.0, 0.6, 2.0)],
                                   shape_extents=[(0.3, 0, 0)], restitution=[0.0]))
    for _ in range(180):
        w.step(DT)
    s = w.read_state()
    x, y = s["position"][first, :2]
    assert x > 2.0  # rolled down-slope (+x)
    surface = -slope * x
    assert y > surface  # stayed above the ramp (never fell through a triangle)
    assert abs((y - surface) * math.cos(math.atan(slope)) - 0.3) < 0.02


def test_mesh_snapshot_resumes(oracle):
    v, t = grid_mesh(6, 6, height=lambda x, z: 0.3 * np.sin(x) * np.cos(z))
    w = world(oracle)
    w.add_triangle_mesh(v, t)
    w.add_bodies(ax.Bodies(type=[1] * 4, shape=[0, 1, 2, 3], position=[(1, 2, 1), (3, 2, 3), (2, 2.5, 4), (4, 3, 1)],
                           shape_extents=[(0.3, 0, 0), (0.3, 0.3, 0.3), (0.2, 0.3, 0), (0.3, 0.2, 0)]))
    for _ in range(60):
        w.step(DT)
    snap = w.save_snapshot()
    r = world(oracle)
    r.load_snapshot(snap)
    for _ in range(40):
        w.step(DT)
        r.step(DT)
    a, b = w.read_state(), r.read_state()
    assert all(np.array_equal(a[k], b[k]) for k in a)


def terrain_scene(lib_world, n=300, seed=9):
    v, t = grid_mesh(20, 20, cell=1.0, height=lambda x, z: 0.4 * np.sin(0.7 * x) * np.cos(0.5 * z))
    lib_world.add_triangle_mesh(v, t, friction=0.6)
    lib_world.add_convex_hull([(x, y, z) for x in (-0.3, 0.3) for y in (-0.3, 0.3) for z in (-0.3, 0.3)])
    rng = np.random.default_rng(seed)
    shapes = rng.choice([ax.SHAPE_SPHERE, ax.SHAPE_BOX, ax.SHAPE_CAPSULE, ax.SHAPE_CYLINDER, ax.SHAPE_CONVEX], n)
    k = np.arange(n)
    pos = np.column_stack([1.5 + (k % 10) * 1.8, 2.0 + (k // 100) * 1.5, 1.5 + ((k // 10) % 10) * 1.8])
    pos += rng.uniform(-0.1, 0.1, (n, 3))
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    ext = np.column_stack([rng.uniform(0.2, 0.4, n), rng.uniform(0.2, 0.4, n), rng.uniform(0.2, 0.4, n)])
    lib_world.add_bodies(ax.Bodies(type=np.ones(n, np.uint32), shape=shapes.astype(np.uint32), position=pos,
                                   rotation=q, shape_extents=ext, convex_hull=np.zeros(n, np.uint32),
                                   friction=np.full(n, 0.6)))


@pytest.mark.gpu
def test_gpu_terrain_bit_exact(gpu_lib, oracle):
    g, o = world(gpu_lib), world(oracle)
    oracle.oracle_set_threads(o.handle, 8)
    terrain_scene(g)
    terrain_scene(o)
    mesh_contacts = 0
    for k in range(150):
        sg, so = g.step(DT), o.step(DT)
        assert (sg.pair_count, sg.manifold_count, sg.contact_point_count) == \
            (so.pair_count, so.manifold_count, so.contact_point_count), k
        a, b = g.read_state(), o.read_state()
        for key in a:
            assert np.array_equal(a[key], b[key]), (k, key)
        if k % 15 == 0:
            cg = ax.canonical_contacts(g.read_contacts())
            co = ax.canonical_contacts(o.read_contacts())
            assert cg.tobytes() == co.tobytes(), k
            mesh_contacts += int((cg["body_a"] < 800).sum())
    assert mesh_contacts > 0
