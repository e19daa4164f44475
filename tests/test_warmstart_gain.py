"""What the trained network gains over the plain previous-step warm start.

Training is reproducible (fixed-order gradient sums), so the measurements below are fixed
for a seed.  First a small network is trained on the GPU from plain-solver samples of
separately seeded tower scenes; on held-out scenes it must predict the converged impulses
better than the previous-step impulses do (the plain warm start is the zero correction).
Then the committed network (axiom-physics-engine_gb300/weights/warmstart_towers.npy,
trained by the project's kernels with warmstart.py) is evaluated on a tower scene seeded
apart from its training scenes and from the benchmark's: both arms resume the same settled
state and solve to the same 1e-4 PGS residual, so the network only changes the number of
sweeps, never the accepted answer.  It must save at least 5 % of the sweeps.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import axiom_gb300 as ax
import warmstart as ws

pytestmark = pytest.mark.gpu

WEIGHTS = Path(ws.__file__).resolve().parent / "weights" / "warmstart_towers.npy"


def test_learned_warm_start_predicts_converged_impulses(gpu_lib):
    f, t = ws.generate_samples(gpu_lib, 400_000, towers=256, seed=2000, steps_per_scene=40)
    params, losses = ws.train_network(gpu_lib, f, t, epochs=8, batch=4096, lr=1e-3)
    assert losses[-1] < losses[0]
    fh, th = ws.generate_samples(gpu_lib, 60_000, towers=128, seed=3000, steps_per_scene=20)
    net = ws.Mlp(gpu_lib, params=params)
    pred = net.forward(fh)
    net.close()
    mse_net = float(np.mean((pred.astype(np.float64) - th) ** 2))
    mse_prev = float(np.mean(th.astype(np.float64) ** 2))
    print(f"\nheld-out MSE of the correction: network {mse_net:.4g}, previous-step start {mse_prev:.4g}")
    assert mse_net < mse_prev


def test_committed_network_saves_sweeps(gpu_lib):
    params = np.load(WEIGHTS).astype(np.float32)
    assert params.shape == (ax.MLP_PARAM_COUNT,)
    ev = ws.evaluate(gpu_lib, params, towers=128, seed=7, steps=8, settle=5)
    plain, learned = ev["plain"], ev["learned"]
    # both reach the threshold (the cap is far above the iterations needed)
    assert plain["max_residual"] <= 1e-4 and learned["max_residual"] <= 1e-4
    print(f"\nplain {plain['mean_iterations']:.0f} sweeps, learned {learned['mean_iterations']:.0f} sweeps, "
          f"reduction {100 * ev['iteration_reduction']:.1f} %, solver time reduction "
          f"{100 * ev['time_reduction']:.1f} %")
    assert ev["iteration_reduction"] >= 0.05
