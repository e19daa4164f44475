"""Body state in and out of a world: axiom_world_read_state / write_state.

The arrays move by bulk copies through device staging regions and one kernel converts the
layout; page-locked (pinned) and pageable host arrays must give the same bytes, for every
subset of the four arrays.
"""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax

pytestmark = pytest.mark.gpu

FIELDS = (("position", 3), ("rotation", 4), ("linear_velocity", 3), ("angular_velocity", 3))


def pinned_like(n):
    import torch

    return {k: torch.empty((n, c), dtype=torch.float32, pin_memory=True).numpy() for k, c in FIELDS}


def test_pinned_and_pageable_state_agree(gpu_lib):
    sc = ax.Scene.mixed(seed=4, count=5000, size=(20.0, 20.0, 20.0), lib=gpu_lib)
    w = ax.PhysicsWorld(ax.default_config(gpu_lib, time_step=1 / 120), lib=gpu_lib)
    w.add_bodies(sc.bodies)
    for _ in range(5):
        w.step(1 / 120)
    n = w.body_count()
    pageable = w.read_state()
    pinned = w.read_state(out=pinned_like(n))
    for k, _ in FIELDS:
        assert np.array_equal(pageable[k], pinned[k]), k
    # write a perturbed state from pinned arrays, read it back through pageable ones
    rng = np.random.default_rng(1)
    src = pinned_like(n)
    for k, c in FIELDS:
        src[k][:] = pageable[k] + rng.normal(scale=0.01, size=(n, c)).astype(np.float32)
    w.write_state(**src)
    back = w.read_state()
    for k, _ in FIELDS:
        assert np.array_equal(back[k], src[k]), k
    # a partial write (velocities only, pageable) leaves the other fields alone
    lin = np.zeros((n, 3), np.float32)
    w.write_state(linear_velocity=lin)
    again = w.read_state(out=pinned_like(n))
    assert np.array_equal(again["linear_velocity"], lin)
    for k in ("position", "rotation", "angular_velocity"):
        assert np.array_equal(again[k], src[k]), k
    # two fresh worlds fed the same state, one from pinned and one from pageable arrays,
    # step identically
    fresh = []
    for src_state in (again, {k: np.array(v) for k, v in again.items()}):
        f = ax.PhysicsWorld(ax.default_config(gpu_lib, time_step=1 / 120), lib=gpu_lib)
        f.add_bodies(sc.bodies)
        f.write_state(**src_state)
        f.step(1 / 120)
        fresh.append(f.read_state())
    for k, _ in FIELDS:
        assert np.array_equal(fresh[0][k], fresh[1][k]), k
