"""What the trained network gains over the plain previous-step warm start.

Trains the warm-start network on the GPU from plain-solver samples of separately seeded
tower scenes, then steps one evaluation scene twice — plain previous-step warm start and
learned warm start — to the same 1e-4 PGS residual.  The accepted answer has the same
residual bound either way; the network may only change the number of sweeps.
"""
from __future__ import annotations

import numpy as np
import pytest

import axiom_gb300 as ax
import warmstart as ws

pytestmark = pytest.mark.gpu


def test_learned_warm_start_needs_fewer_sweeps(gpu_lib):
    f, t = ws.generate_samples(gpu_lib, 400_000, towers=256, seed=2000, steps_per_scene=40)
    params, losses = ws.train_network(gpu_lib, f, t, epochs=8, batch=4096, lr=1e-3)
    assert losses[-1] < losses[0]
    ev = ws.evaluate(gpu_lib, params, towers=96, seed=7, steps=20, settle=5)
    plain, learned = ev["plain"], ev["learned"]
    # both reach the threshold (the cap is far above the iterations needed)
    assert plain["max_residual"] <= 1e-4 and learned["max_residual"] <= 1e-4
    print(f"\nplain {plain['mean_iterations']:.0f} sweeps, learned {learned['mean_iterations']:.0f} sweeps, "
          f"reduction {100 * ev['iteration_reduction']:.1f} %, solver time reduction "
          f"{100 * ev['time_reduction']:.1f} %")
    assert learned["mean_iterations"] < plain["mean_iterations"]
