"""Pins the oracle's math and the scene RNG to the reference.

Golden vectors in tests/golden/ref_math.json were computed by the reference's own
headers (include/axiom/math/{random,aabb,vec3}.hpp), see tests/golden/make_golden.py.
Quaternion cases restate the reference's tests/math/quat_test.cpp and
transform_test.cpp expectations (their GLM-backed implementation cannot be built here).
"""
from __future__ import annotations

import ctypes
import json
import math

import numpy as np
import pytest

from conftest import ROOT

GOLD = json.loads((ROOT / "tests" / "golden" / "ref_math.json").read_text())
F = ctypes.POINTER(ctypes.c_float)


def fa(values):
    return (ctypes.c_float * len(values))(*values)


def f32(x):
    return float(np.float32(x))


# ---- DeterministicRNG (random.hpp:19-64; random_test.cpp:15-59) ----
@pytest.mark.parametrize("case", GOLD["rng"], ids=lambda c: f"seed{c['seed']}")
def test_rng_matches_reference_sequence(lib, case):
    n = len(case["u32"])
    out = np.empty(n, np.uint32)
    lib.axiom_rng_u32(case["seed"], n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    assert out.tolist() == case["u32"]
    fl = np.empty(len(case["float"]), np.float32)
    lib.axiom_rng_float(case["seed"], len(fl), fl.ctypes.data_as(F))
    assert fl.tolist() == [f32(v) for v in case["float"]]
    jit = np.empty(len(case["float_jitter"]), np.float32)
    lib.axiom_rng_float_range(case["seed"], len(jit), -0.002, 0.002, jit.ctypes.data_as(F))
    assert jit.tolist() == [f32(v) for v in case["float_jitter"]]
    r = np.empty(len(case["float_10_20"]), np.float32)
    lib.axiom_rng_float_range(case["seed"], len(r), 10.0, 20.0, r.ctypes.data_as(F))
    assert r.tolist() == [f32(v) for v in case["float_10_20"]]


def test_rng_same_seed_same_sequence_and_range(lib):
    a = np.empty(1000, np.uint32)
    b = np.empty(1000, np.uint32)
    lib.axiom_rng_u32(12345, 1000, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    lib.axiom_rng_u32(12345, 1000, b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    assert (a == b).all() and len(set(a.tolist())) > 900
    f = np.empty(1000, np.float32)
    lib.axiom_rng_float(42, 1000, f.ctypes.data_as(F))
    assert (f >= 0).all() and (f < 1).all()


# ---- AABB (aabb.hpp:132-215; aabb_test.cpp:179-208) ----
def test_aabb_intersects_matches_reference(oracle):
    for c in GOLD["aabb"]:
        amin, amax = fa([0.0] * 3), fa([0.0] * 3)
        bmin, bmax = fa([0.0] * 3), fa([0.0] * 3)
        oracle.oracle_aabb_from_center(fa(c["ca"]), fa(c["ea"]), 0.0, amin, amax)
        oracle.oracle_aabb_from_center(fa(c["cb"]), fa(c["eb"]), 0.0, bmin, bmax)
        assert list(amin) == [f32(v) for v in c["amin"]]
        assert list(amax) == [f32(v) for v in c["amax"]]
        assert bool(oracle.oracle_aabb_intersects(amin, amax, bmin, bmax)) == c["ab"]
        assert bool(oracle.oracle_aabb_intersects(bmin, bmax, amin, amax)) == c["ba"]
        mmin, mmax = fa([0.0] * 3), fa([0.0] * 3)
        oracle.oracle_aabb_from_center(fa(c["ca"]), fa(c["ea"]), c["margin"], mmin, mmax)
        # expand(margin) after fromCenterExtents equals centre -/+ (extent + margin) on
        # this quarter grid (all values exact in fp32)
        assert list(mmin) == [f32(v) for v in c["am_min"]]
        assert list(mmax) == [f32(v) for v in c["am_max"]]


def test_aabb_reference_test_cases(oracle):
    def box(lo, hi):
        return fa(lo), fa(hi)
    a = box([0, 0, 0], [2, 2, 2]); b = box([1, 1, 1], [3, 3, 3])
    assert oracle.oracle_aabb_intersects(*a, *b) and oracle.oracle_aabb_intersects(*b, *a)
    a = box([0, 0, 0], [1, 1, 1]); b = box([1, 0, 0], [2, 1, 1])
    assert oracle.oracle_aabb_intersects(*a, *b)  # touching counts
    b = box([2, 0, 0], [3, 1, 1])
    assert not oracle.oracle_aabb_intersects(*a, *b) and not oracle.oracle_aabb_intersects(*b, *a)
    outer = box([0, 0, 0], [4, 4, 4]); inner = box([1, 1, 1], [3, 3, 3])
    assert oracle.oracle_aabb_intersects(*outer, *inner) and oracle.oracle_aabb_intersects(*inner, *outer)


def test_vec3_ops_match_reference(oracle):
    for c in GOLD["vec3"]:
        d = ctypes.c_float()
        cr, nz = fa([0.0] * 3), fa([0.0] * 3)
        oracle.oracle_vec3_ops(fa(c["a"]), fa(c["b"]), ctypes.byref(d), cr, nz)
        assert d.value == f32(c["dot"])
        assert list(cr) == [f32(v) for v in c["cross"]]
        assert list(nz) == [f32(v) for v in c["normalized"]]
    assert GOLD["vec3"][0]["normalized"] == [0, 0, 0]  # zero vector normalises to zero


# ---- Quaternion restatement (quat_test.cpp:166-229, transform_test.cpp:257-290) ----
def rot(oracle, q, v):
    out = fa([0.0] * 3)
    oracle.oracle_quat_rotate(fa(q), fa(v), out)
    return list(out)


def axis_angle(oracle, axis, ang):
    out = fa([0.0] * 4)
    oracle.oracle_quat_from_axis_angle(fa(axis), ang, out)
    return list(out)


def close(a, b, eps=1e-5):
    return all(abs(x - y) < eps for x, y in zip(a, b))


def test_quat_vector_rotation_180_about_z(oracle):
    q = axis_angle(oracle, [0, 0, 1], math.pi)
    assert close(rot(oracle, q, [1, 0, 0]), [-1, 0, 0])


def test_quat_multiplication_order(oracle):
    qz = axis_angle(oracle, [0, 0, 1], math.pi / 2)
    qx = axis_angle(oracle, [1, 0, 0], math.pi / 2)
    comb = fa([0.0] * 4)
    oracle.oracle_quat_mul(fa(qx), fa(qz), comb)  # apply qz first, then qx
    assert close(rot(oracle, list(comb), [1, 0, 0]), [0, 0, 1])


def test_quat_inverse_product_is_identity(oracle):
    q = axis_angle(oracle, [0, 0, 1], math.pi / 4)
    inv = [-q[0], -q[1], -q[2], q[3]]
    out = fa([0.0] * 4)
    oracle.oracle_quat_mul(fa(q), fa(inv), out)
    assert close(list(out), [0, 0, 0, 1])


def test_quat_normalize(oracle):
    out = fa([0.0] * 4)
    oracle.oracle_quat_normalize(fa([1.0, 2.0, 2.0, 0.0]), out)
    assert abs(math.sqrt(sum(v * v for v in out)) - 1.0) < 1e-5


def test_transform_point_rotation(oracle):
    q = axis_angle(oracle, [0, 0, 1], math.pi / 2)
    assert close(rot(oracle, q, [1, 0, 0]), [0, 1, 0])
    ident = [0, 0, 0, 1]
    assert rot(oracle, ident, [1, 2, 3]) == [1, 2, 3]  # identity is exact
