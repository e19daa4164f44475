"""The oracle's narrowphase against closed-form answers and an independent SAT check.

The reference has no narrowphase to compare with (its collision layer is empty), so the
oracle's contact generation is checked here on configurations with known answers, and its
GJK/EPA penetration depth against a separating-axis computation in numpy.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import pytest

import axiom_gb300 as ax

F = ctypes.POINTER(ctypes.c_float)
IDENT = [0.0, 0.0, 0.0, 1.0]


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


def rotmat(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def sat_depth(pa, qa, ea, pb, qb, eb):
    """Minimum overlap over the 15 OBB separating axes, and that axis."""
    A, B = rotmat(qa), rotmat(qb)
    T = np.asarray(pb, float) - np.asarray(pa, float)
    axes = [A[:, i] for i in range(3)] + [B[:, i] for i in range(3)]
    for i in range(3):
        for j in range(3):
            c = np.cross(A[:, i], B[:, j])
            if np.linalg.norm(c) > 1e-6:
                axes.append(c / np.linalg.norm(c))
    best, bax = np.inf, None
    for L in axes:
        ra = sum(ea[i] * abs(A[:, i] @ L) for i in range(3))
        rb = sum(eb[i] * abs(B[:, i] @ L) for i in range(3))
        ov = ra + rb - abs(T @ L)
        if ov < best:
            best, bax = ov, L * (1.0 if T @ L >= 0 else -1.0)
    return best, bax


def test_sphere_on_box_top(collide):
    k, n, p, d = collide(ax.SHAPE_SPHERE, [0, 1.4, 0], IDENT, [0.5, 0, 0],
                         ax.SHAPE_BOX, [0, 0, 0], IDENT, [1, 1, 1])
    assert k == 1 and np.allclose(n, [0, -1, 0]) and abs(d[0] - 0.1) < 1e-6
    assert np.allclose(p[0], [0, 0.95, 0], atol=1e-6)
    # swapped order flips the normal, keeps the point
    k2, n2, p2, d2 = collide(ax.SHAPE_BOX, [0, 0, 0], IDENT, [1, 1, 1],
                             ax.SHAPE_SPHERE, [0, 1.4, 0], IDENT, [0.5, 0, 0])
    assert k2 == 1 and np.allclose(n2, -n) and np.allclose(p2, p) and np.allclose(d2, d)


def test_sphere_inside_box_pushes_through_nearest_face(collide):
    k, n, p, d = collide(ax.SHAPE_SPHERE, [0.8, 0.1, 0], IDENT, [0.3, 0, 0],
                         ax.SHAPE_BOX, [0, 0, 0], IDENT, [1, 1, 1])
    assert k == 1 and np.allclose(n, [-1, 0, 0]) and abs(d[0] - 0.5) < 1e-6


def test_box_resting_on_plane_gives_four_points(collide):
    k, n, p, d = collide(ax.SHAPE_BOX, [2, 0.49, -1], IDENT, [0.5, 0.5, 0.5],
                         ax.SHAPE_PLANE, [0, 0, 0], IDENT, [0, 0, 0])
    assert k == 4 and np.allclose(n, [0, 1, 0])
    assert np.allclose(d, 0.01, atol=1e-6)
    assert np.allclose(sorted(p[:, 0]), [1.5, 1.5, 2.5, 2.5]) and np.allclose(p[:, 1], -0.005, atol=1e-6)


def test_tilted_box_on_plane_deepest_first(collide):
    q = quat_axis_angle([0, 0, 1], 0.3)
    k, n, p, d = collide(ax.SHAPE_BOX, [0, 0.5, 0], q, [0.5, 0.5, 0.5],
                         ax.SHAPE_PLANE, [0, 0, 0], IDENT, [0, 0, 0])
    assert k == 2 and np.all(np.diff(d) <= 0)


def test_stacked_boxes_face_manifold(collide):
    k, n, p, d = collide(ax.SHAPE_BOX, [0, 0, 0], IDENT, [0.5, 0.5, 0.5],
                         ax.SHAPE_BOX, [0.1, 0.99, 0.05], IDENT, [0.5, 0.5, 0.5])
    assert k == 4 and np.allclose(n, [0, 1, 0], atol=1e-6)
    assert np.allclose(d, 0.01, atol=1e-5)
    assert np.allclose(p[:, 1], 0.495, atol=1e-5)


@pytest.mark.parametrize("seed", range(16))
def test_box_box_epa_depth_matches_sat(collide, seed):
    """Shallow random overlaps: the normal follows the SAT axis and the deepest point's
    depth equals the SAT penetration."""
    rng = np.random.default_rng(seed)
    ea = rng.uniform(0.2, 0.8, 3).tolist()
    eb = rng.uniform(0.2, 0.8, 3).tolist()
    qa = quat_axis_angle(rng.normal(size=3), rng.uniform(0, math.pi))
    qb = quat_axis_angle(rng.normal(size=3), rng.uniform(0, math.pi))
    dirn = rng.normal(size=3)
    dirn /= np.linalg.norm(dirn)
    lo, hi = 0.0, 4.0  # bisect the distance at which the boxes just touch
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if sat_depth([0, 0, 0], qa, ea, (dirn * mid).tolist(), qb, eb)[0] > 0:
            lo = mid
        else:
            hi = mid
    pb = (dirn * (lo - rng.uniform(0.005, 0.05))).tolist()
    depth, axis = sat_depth([0, 0, 0], qa, ea, pb, qb, eb)
    k, n, p, d = collide(ax.SHAPE_BOX, [0, 0, 0], qa, ea, ax.SHAPE_BOX, pb, qb, eb)
    assert k >= 1 and depth > 0
    assert abs(np.linalg.norm(n) - 1) < 1e-5
    assert float(n @ axis) > 0.99, (n, axis)
    assert abs(float(d.max()) - depth) < 2e-3, (d, depth)


def test_separated_boxes(collide):
    k, *_ = collide(ax.SHAPE_BOX, [0, 0, 0], IDENT, [0.5, 0.5, 0.5],
                    ax.SHAPE_BOX, [1.2, 0, 0], quat_axis_angle([1, 1, 0], 0.4), [0.5, 0.5, 0.5])
    assert k == 0


def test_capsule_lying_on_box_two_points(collide):
    q = quat_axis_angle([0, 0, 1], math.pi / 2)  # axis along x
    k, n, p, d = collide(ax.SHAPE_BOX, [0, 0, 0], IDENT, [1, 0.5, 1],
                         ax.SHAPE_CAPSULE, [0, 0.69, 0], q, [0.2, 0.4, 0])
    assert k == 2 and np.allclose(n, [0, 1, 0], atol=1e-5)
    assert np.allclose(d, 0.01, atol=1e-5)
    assert np.allclose(sorted(p[:, 0]), [-0.4, 0.4], atol=1e-5)


def test_capsule_capsule_crossing(collide):
    qx = quat_axis_angle([0, 0, 1], math.pi / 2)
    qz = quat_axis_angle([1, 0, 0], math.pi / 2)
    k, n, p, d = collide(ax.SHAPE_CAPSULE, [0, 0, 0], qx, [0.2, 1.0, 0],
                         ax.SHAPE_CAPSULE, [0, 0.35, 0], qz, [0.2, 1.0, 0])
    assert k == 1 and np.allclose(n, [0, 1, 0], atol=1e-6) and abs(d[0] - 0.05) < 1e-6


def test_sphere_capsule_and_capsule_plane(collide):
    k, n, p, d = collide(ax.SHAPE_SPHERE, [0.3, 1.3, 0], IDENT, [0.3, 0, 0],
                         ax.SHAPE_CAPSULE, [0, 0, 0], IDENT, [0.2, 1.0, 0])
    assert k == 1 and abs(d[0] - (0.5 - math.hypot(0.3, 0.3))) < 1e-6
    q = quat_axis_angle([0, 0, 1], math.pi / 2)
    k, n, p, d = collide(ax.SHAPE_CAPSULE, [0, 0.19, 0], q, [0.2, 0.5, 0],
                         ax.SHAPE_PLANE, [0, 0, 0], IDENT, [0, 0, 0])
    assert k == 2 and np.allclose(d, 0.01, atol=1e-6) and np.allclose(n, [0, 1, 0])


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("overlap", [0.001, 0.004, 0.1])
def test_box_box_exactly_aligned_stack(collide, axis, overlap):
    # two identical boxes face to face on one axis: the origin of the Minkowski difference
    # lies on GJK's first segment, where the usual search direction is the zero vector;
    # the contact must still be the full face with the overlap as depth
    he = 0.5
    pb = [0.0, 0.0, 0.0]
    pb[axis] = 2 * he - overlap
    k, n, p, d = collide(ax.SHAPE_BOX, [0, 0, 0], IDENT, [he, he, he], ax.SHAPE_BOX, pb, IDENT, [he, he, he])
    expect_n = np.zeros(3)
    expect_n[axis] = 1.0
    sat, _ = sat_depth([0, 0, 0], IDENT, [he] * 3, pb, IDENT, [he] * 3)
    assert k == 4 and np.allclose(n, expect_n)
    assert np.allclose(d, sat, rtol=1e-3, atol=2e-6)
