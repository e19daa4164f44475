"""Body validation at the boundary: a body with a non-finite number, a zero-length
rotation or a negative mass property is an invalid rigid body (core::ErrorCode
InvalidRigidBody, include/axiom/core/error_code.hpp:41), and nothing of the call is added.

The CPU tests drive the oracle (which validates with the same rules); the GPU test drives
the CUDA library."""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax


def _spheres(n=4):
    return dict(type=np.full(n, ax.BODY_DYNAMIC, np.uint32), shape=np.full(n, ax.SHAPE_SPHERE, np.uint32),
                position=np.arange(3 * n, dtype=np.float32).reshape(n, 3), shape_extents=np.full((n, 3), 0.5, np.float32))


BAD = [
    ("position", lambda f: f["position"].__setitem__((2, 1), np.nan)),
    ("position", lambda f: f["position"].__setitem__((1, 0), np.inf)),
    ("rotation", lambda f: f.__setitem__("rotation", np.tile(np.float32([0, 0, 0, 1]), (4, 1)))
     or f["rotation"].__setitem__(3, 0.0)),
    ("rotation", lambda f: f.__setitem__("rotation", np.tile(np.float32([0, 0, 0, 1]), (4, 1)))
     or f["rotation"].__setitem__((0, 2), np.nan)),
    ("linear_velocity", lambda f: f.__setitem__("linear_velocity", np.zeros((4, 3), np.float32))
     or f["linear_velocity"].__setitem__((3, 2), -np.inf)),
    ("angular_velocity", lambda f: f.__setitem__("angular_velocity", np.zeros((4, 3), np.float32))
     or f["angular_velocity"].__setitem__((0, 0), np.nan)),
    ("mass", lambda f: f.__setitem__("mass", np.float32([1, 2, -1, 3]))),
    ("mass", lambda f: f.__setitem__("mass", np.float32([1, np.nan, 1, 3]))),
    ("inertia", lambda f: f.__setitem__("inertia", np.ones((4, 3), np.float32))
     or f["inertia"].__setitem__((1, 1), -2.0)),
    ("density", lambda f: f.__setitem__("density", np.float32([1000, 1000, np.inf, 1000]))),
    ("friction", lambda f: f.__setitem__("friction", np.float32([0.5, -0.1, 0.5, 0.5]))),
    ("restitution", lambda f: f.__setitem__("restitution", np.float32([0.5, 0.5, 0.5, np.nan]))),
    ("linear_damping", lambda f: f.__setitem__("linear_damping", np.float32([0, 0, -1, 0]))),
    ("angular_damping", lambda f: f.__setitem__("angular_damping", np.float32([np.nan, 0, 0, 0]))),
    ("shape_extents", lambda f: f["shape_extents"].__setitem__((0, 0), np.inf)),
    ("rolling_friction", lambda f: f.__setitem__("rolling_friction", np.float32([0, 0.1, -0.2, 0]))),
]


def test_oracle_rolling_friction_is_carried(oracle):
    """MaterialInfo::rollingFriction travels with the body into snapshots and back."""
    f = _spheres()
    f["rolling_friction"] = np.float32([0.0, 0.05, 0.1, 0.25])
    w = ax.PhysicsWorld(ax.default_config(oracle), lib=oracle)
    w.add_bodies(ax.Bodies(**f))
    _, bodies, _, _ = ax.parse_snapshot(w.save_snapshot())
    assert np.array_equal(bodies["rolling_friction"], f["rolling_friction"])
    assert (bodies["reserved"] == 0).all()
    r = ax.PhysicsWorld(ax.default_config(oracle), lib=oracle)
    r.load_snapshot(w.save_snapshot())
    assert r.save_snapshot() == w.save_snapshot()


def _check_rejects(lib):
    for field, spoil in BAD:
        f = _spheres()
        spoil(f)
        w = ax.PhysicsWorld(ax.default_config(lib), lib=lib)
        with pytest.raises(ax.AxiomError) as e:
            w.add_bodies(ax.Bodies(**f))
        assert e.value.code == ax.ERR_INVALID_RIGID_BODY, (field, e.value.code)
        assert w.body_count() == 0, field
        # a valid description is still accepted afterwards
        w.add_bodies(ax.Bodies(**_spheres()))
        assert w.body_count() == 4
        w.close()


def test_oracle_rejects_non_finite_bodies(oracle):
    _check_rejects(oracle)


@pytest.mark.gpu
def test_gpu_rejects_non_finite_bodies(gpu_lib):
    _check_rejects(gpu_lib)
