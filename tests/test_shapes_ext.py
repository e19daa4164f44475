"""Cylinders and convex hulls (gui::ShapeType::Cylinder / Convex,
include/axiom/gui/body_inspector.hpp:20-27).

The oracle's contacts are checked on configurations with closed-form answers (a cylinder
standing or lying on a plane, a sphere against cap and side, a box on a cap, a hull made of
a box's corners against a box) and the GPU step is compared with the oracle bit for bit on
mixed scenes that contain every new pair type.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import pytest

import axiom_gb300 as ax

F = ctypes.POINTER(ctypes.c_float)
IDENT = [0.0, 0.0, 0.0, 1.0]
CUBE = [(x, y, z) for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)]


@pytest.fixture(scope="module")
def collide(oracle):
    fn = oracle.oracle_collide_shapes
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, F, F, F, ctypes.c_uint32, F, F, F, F, F, F]

    def run(sa, pa, qa, ea, sb, pb, qb, eb):
        n = (ctypes.c_float * 3)()
        p = (ctypes.c_float * 12)()
        d = (ctypes.c_float * 4)()
        fa = lambda v: (ctypes.c_float * len(v))(*v)
        k = fn(sa, fa(pa), fa(qa), fa(ea), sb, fa(pb), fa(qb), fa(eb), n, p, d)
        return k, np.array(n[:]), np.array(p[:]).reshape(4, 3)[:k], np.array(d[:k])
    return run


def quat_axis_angle(axis, ang):
    a = np.asarray(axis, float)
    a = a / np.linalg.norm(a)
    s = math.sin(ang / 2)
    return [a[0] * s, a[1] * s, a[2] * s, math.cos(ang / 2)]


def test_cylinder_standing_on_plane(collide):
    # axis up, sunk 0.01: four rim points of the bottom cap at the same depth
    k, n, p, d = collide(ax.SHAPE_CYLINDER, [0, 0.49, 0], IDENT, [0.5, 0.5, 0], ax.SHAPE_PLANE, [0, 0, 0], IDENT,
                         [0, 0, 0])
    assert k == 4 and np.allclose(n, [0, 1, 0])
    assert np.allclose(d, 0.01, atol=1e-6)
    assert np.allclose(np.hypot(p[:, 0], p[:, 2]), 0.5, atol=1e-6)
    assert np.allclose(p[:, 1], -0.005, atol=1e-6)


def test_cylinder_lying_on_plane(collide):
    q = quat_axis_angle([0, 0, 1], math.pi / 2)  # axis along x
    k, n, p, d = collide(ax.SHAPE_CYLINDER, [0, 0.49, 0], q, [0.5, 0.8, 0], ax.SHAPE_PLANE, [0, 0, 0], IDENT,
                         [0, 0, 0])
    assert k == 2 and np.allclose(d, 0.01, atol=1e-6)
    assert np.allclose(sorted(p[:, 0]), [-0.8, 0.8], atol=1e-6) and np.allclose(p[:, 2], 0.0, atol=1e-6)


@pytest.mark.parametrize("where, expect_n, depth", [
    ([0.0, 1.0, 0.0], [0, -1, 0], 0.1),     # above the cap
    ([0.7, 0.0, 0.0], [-1, 0, 0], 0.1),     # beside the side
    ([0.7, 0.95, 0.0], None, None),         # off the rim edge
    ([0.0, 0.7, 0.0], [0, -1, 0], 0.4),     # centre inside, nearer the cap than the side
])
def test_sphere_cylinder(collide, where, expect_n, depth):
    # cylinder r 0.5, half-height 0.8 along y; sphere r 0.3 (normal sphere -> cylinder)
    k, n, p, d = collide(ax.SHAPE_SPHERE, where, IDENT, [0.3, 0, 0], ax.SHAPE_CYLINDER, [0, 0, 0], IDENT,
                         [0.5, 0.8, 0])
    if expect_n is None:
        dist = math.hypot(0.7 - 0.5, 0.95 - 0.8)
        assert k == 1 and abs(d[0] - (0.3 - dist)) < 1e-6
        assert np.allclose(n, -np.array([0.2, 0.15, 0]) / dist, atol=1e-6)
    else:
        assert k == 1 and np.allclose(n, expect_n, atol=1e-6) and abs(d[0] - depth) < 1e-6


def test_box_on_cylinder_cap(collide):
    # unit box resting 0.02 deep on a wide cylinder's cap: four box corners, normal along the axis
    k, n, p, d = collide(ax.SHAPE_CYLINDER, [0, 0, 0], IDENT, [2.0, 0.5, 0], ax.SHAPE_BOX, [0.1, 0.98, 0.2],
                         IDENT, [0.5, 0.5, 0.5])
    assert k == 4 and np.allclose(n, [0, 1, 0], atol=1e-5)
    assert np.allclose(d, 0.02, atol=1e-4)


def test_cylinder_stacked_on_cylinder(collide):
    k, n, p, d = collide(ax.SHAPE_CYLINDER, [0, 0, 0], IDENT, [0.5, 0.5, 0], ax.SHAPE_CYLINDER, [0.05, 0.99, 0],
                         IDENT, [0.5, 0.5, 0])
    assert k == 4 and np.allclose(n, [0, 1, 0], atol=1e-5)
    assert np.allclose(d, 0.01, atol=1e-4)


def hull_world(lib, **cfg):
    c = dict(time_step=1 / 120, velocity_iterations=10)
    c.update(cfg)
    w = ax.PhysicsWorld(ax.default_config(lib, **c), lib=lib)
    hid = w.add_convex_hull(CUBE)
    return w, hid


def test_hull_of_cube_matches_box(lib, oracle):
    # a hull made of a cube's eight corners resting on a box behaves like the box itself
    results = []
    for convex in (False, True):
        w, hid = hull_world(oracle, gravity=(0, 0, 0))
        top = dict(type=[1], shape=[ax.SHAPE_CONVEX if convex else ax.SHAPE_BOX], position=[(0.1, 0.99, -0.05)],
                   shape_extents=[(0.5, 0.5, 0.5)], convex_hull=[hid])
        w.add_bodies(ax.Bodies(type=[0], shape=[ax.SHAPE_BOX], position=[(0, 0, 0)], shape_extents=[(1, 0.5, 1)]))
        w.add_bodies(ax.Bodies(**top))
        st = w.step(1 / 120)
        c = w.read_contacts()
        results.append((st.contact_point_count, c))
    (n0, c0), (n1, c1) = results
    assert n0 == n1 == 4
    assert np.allclose(np.abs(c1["normal"]), [0, 1, 0], atol=1e-5)
    assert np.allclose(c1["penetration_depth"], c0["penetration_depth"], atol=1e-5)


def test_hull_and_cylinder_mass_properties(lib, oracle):
    w, hid = hull_world(oracle)
    w.add_bodies(ax.Bodies(type=[1, 1], shape=[ax.SHAPE_CYLINDER, ax.SHAPE_CONVEX], position=[(0, 2, 0), (3, 2, 0)],
                           shape_extents=[(0.5, 1.0, 0), (0, 0, 0)], convex_hull=[0, hid]))
    _, bodies, _, hulls = ax.parse_snapshot(w.save_snapshot())
    r, h = 0.5, 1.0
    m = 1000.0 * math.pi * r * r * 2 * h
    assert bodies["inv_mass"][0] == pytest.approx(1 / m, rel=1e-6)
    assert bodies["inv_inertia"][0] == pytest.approx([12 / (m * (3 * r * r + 4 * h * h)), 2 / (m * r * r),
                                                      12 / (m * (3 * r * r + 4 * h * h))], rel=1e-5)
    mc = 1000.0  # unit cube
    assert bodies["inv_mass"][1] == pytest.approx(1 / mc, rel=1e-6)
    assert bodies["inv_inertia"][1] == pytest.approx([6 / mc] * 3, rel=1e-5)
    assert len(hulls) == 1 and np.array_equal(hulls[0], np.array(CUBE, np.float32))


def test_hull_validation(lib, oracle):
    w, _ = hull_world(oracle)
    with pytest.raises(ax.AxiomError):
        w.add_convex_hull(CUBE[:3])  # fewer than 4 points
    with pytest.raises(ax.AxiomError):
        w.add_convex_hull(np.zeros((65, 3)) + 1.0)
    with pytest.raises(ax.AxiomError) as e:
        w.add_bodies(ax.Bodies(type=[1], shape=[ax.SHAPE_CONVEX], position=[(0, 0, 0)], shape_extents=[(0, 0, 0)],
                               convex_hull=[7]))
    assert e.value.code == 300


def extended_scene(seed=21, n=400, span=8.0, grid=False):
    """Ground plane + a seeded jumble of spheres, boxes, capsules, cylinders and hulls:
    overlapping at random positions, or (grid) separated on a jittered 2 m grid."""
    rng = np.random.default_rng(seed)
    shapes = rng.choice([ax.SHAPE_SPHERE, ax.SHAPE_BOX, ax.SHAPE_CAPSULE, ax.SHAPE_CYLINDER, ax.SHAPE_CONVEX], n)
    if grid:
        k = np.arange(n)
        side = int(math.ceil(math.sqrt(n / 3)))
        pos = np.column_stack([(k % side) * 2.0, 1.2 + (k // (side * side)) * 2.0, ((k // side) % side) * 2.0])
        pos += rng.uniform(-0.1, 0.1, (n, 3))
    else:
        pos = np.column_stack([rng.uniform(-span, span, n), rng.uniform(0.6, 10.0, n), rng.uniform(-span, span, n)])
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    ext = np.column_stack([rng.uniform(0.2, 0.5, n), rng.uniform(0.2, 0.5, n), rng.uniform(0.2, 0.5, n)])
    hull = rng.integers(0, 2, n).astype(np.uint32)
    t = np.concatenate([[ax.BODY_STATIC], np.full(n, ax.BODY_DYNAMIC)]).astype(np.uint32)
    s = np.concatenate([[ax.SHAPE_PLANE], shapes]).astype(np.uint32)
    return ax.Bodies(type=t, shape=s, position=np.vstack([[0, 0, 0], pos]), rotation=np.vstack([IDENT, q]),
                     shape_extents=np.vstack([[0, 0, 0], ext]), convex_hull=np.concatenate([[0], hull]),
                     friction=np.full(n + 1, 0.6))


def octahedron(s=0.45):
    return [(s, 0, 0), (-s, 0, 0), (0, s, 0), (0, -s, 0), (0, 0, s), (0, 0, -s)]


def make_ext_world(lib, bodies, **cfg):
    c = dict(time_step=1 / 120, velocity_iterations=10)
    c.update(cfg)
    w = ax.PhysicsWorld(ax.default_config(lib, **c), lib=lib)
    w.add_convex_hull(CUBE)
    w.add_convex_hull(octahedron())
    w.add_bodies(bodies)
    return w


def test_oracle_extended_scene_settles(lib, oracle):
    # separated bodies dropped in three layers: they land, pile and come to rest (spheres,
    # capsules and cylinders on their side may keep rolling: there is no rolling friction)
    b = extended_scene(n=150, grid=True)
    w = make_ext_world(oracle, b)
    for _ in range(480):
        st = w.step(1 / 120)
    s = w.read_state()
    assert np.isfinite(s["position"]).all()
    assert (s["position"][1:, 1] > -0.05).all()  # nothing fell through the ground
    assert np.linalg.norm(s["linear_velocity"], axis=1).max() < 5.0
    assert st.manifold_count > 0


@pytest.mark.parametrize("shape, hull, ext, rest_y", [
    (ax.SHAPE_CYLINDER, 0, (0.4, 0.3, 0.0), 0.3),       # upright on its cap
    (ax.SHAPE_CONVEX, 0, (0.0, 0.0, 0.0), 0.5),         # the cube hull on a face
    (ax.SHAPE_CONVEX, 1, (0.0, 0.0, 0.0), 0.45 / math.sqrt(3.0)),  # the octahedron on a face
])
def test_oracle_single_body_comes_to_rest(lib, oracle, shape, hull, ext, rest_y):
    # dropped alone from 1 m with a small tilt: it lands, settles on its face, and stays
    q = quat_axis_angle([1, 0, 1], 0.05 if shape != ax.SHAPE_CONVEX or hull == 0 else 0.9553 + 0.05)
    b = ax.Bodies(type=[0, 1], shape=[ax.SHAPE_PLANE, shape], position=[(0, 0, 0), (0, 1.0, 0)],
                  rotation=[IDENT, q], shape_extents=[(0, 0, 0), ext], convex_hull=[0, hull], friction=[0.6, 0.6],
                  restitution=[0.0, 0.0])
    w = make_ext_world(oracle, b)
    for _ in range(600):
        st = w.step(1 / 120)
    s = w.read_state()
    assert np.linalg.norm(s["linear_velocity"][1]) < 1e-3 and np.linalg.norm(s["angular_velocity"][1]) < 1e-2
    # resting height: the Baumgarte bias leaves about the linear slop (5 mm) of penetration
    assert abs(s["position"][1, 1] - rest_y) < 8e-3
    assert st.contact_point_count >= 3


@pytest.mark.gpu
def test_gpu_extended_shapes_bit_exact(gpu_lib, oracle):
    b = extended_scene()
    g, o = make_ext_world(gpu_lib, b), make_ext_world(oracle, b)
    oracle.oracle_set_threads(o.handle, 8)
    seen = set()
    for k in range(150):
        sg, so = g.step(1 / 120), o.step(1 / 120)
        assert (sg.pair_count, sg.manifold_count, sg.contact_point_count) == \
            (so.pair_count, so.manifold_count, so.contact_point_count), k
        a, c = g.read_state(), o.read_state()
        for key in a:
            assert np.array_equal(a[key], c[key]), (k, key)
        if k % 10 == 0:
            cg = ax.canonical_contacts(g.read_contacts())
            co = ax.canonical_contacts(o.read_contacts())
            assert cg.tobytes() == co.tobytes(), k
            shapes = b.arrays["shape"]
            seen |= {tuple(sorted((int(shapes[x]), int(shapes[y])))) for x, y in zip(cg["body_a"], cg["body_b"])}
    # every new pair type was exercised
    for pair in [(0, 3), (1, 3), (2, 3), (3, 3), (0, 5), (1, 5), (3, 5), (5, 5), (3, 6), (5, 6)]:
        assert pair in seen, pair


@pytest.mark.gpu
def test_gpu_cylinder_stack_bit_exact(gpu_lib, oracle):
    n = 6
    b = ax.Bodies(type=[0] + [1] * n, shape=[ax.SHAPE_PLANE] + [ax.SHAPE_CYLINDER] * n,
                  position=[(0, 0, 0)] + [(0.01 * k, 0.4 + 0.79 * k, 0) for k in range(n)],
                  shape_extents=[(0, 0, 0)] + [(0.5, 0.4, 0)] * n, friction=[0.6] * (n + 1))
    g, o = make_ext_world(gpu_lib, b), make_ext_world(oracle, b)
    for k in range(240):
        g.step(1 / 120)
        o.step(1 / 120)
        a, c = g.read_state(), o.read_state()
        assert all(np.array_equal(a[key], c[key]) for key in a), k
    top = a["position"][-1]
    assert abs(top[1] - (0.4 + 0.8 * (n - 1))) < 0.05  # the stack still stands
