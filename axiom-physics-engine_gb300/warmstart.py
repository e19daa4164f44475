"""Learned PGS warm start: data generation, training and evaluation on the GPU.

The network (14 -> 128 -> 128 -> 128 -> 3, SiLU; see include/axiom_c.h) predicts, from
per-contact features, the correction that takes the previous-step impulses to the
converged ones; PGS then starts from previous + correction.  Training samples come from the
plain solver itself: tower scenes stepped with the previous-step warm start in
residual-tolerance mode, recording (features, final impulses) at every step.  The trained
network is then used as the warm start of the same solver on separately seeded scenes;
the solver still iterates to the same residual, so only the iteration count changes.

    python axiom-physics-engine_gb300/warmstart.py --samples 5000000 --towers 2048
"""
from __future__ import annotations

import argparse
import ctypes
import json
import sys
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
import axiom_gb300 as ax  # noqa: E402

PARAM_COUNT = ax.MLP_PARAM_COUNT
OFF_W1, OFF_B1 = 0, 128 * 16
OFF_W2 = OFF_B1 + 128
OFF_B2 = OFF_W2 + 128 * 128
OFF_W3 = OFF_B2 + 128
OFF_B3 = OFF_W3 + 128 * 128
OFF_W4 = OFF_B3 + 128
OFF_B4 = OFF_W4 + 3 * 128


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation; the two padding inputs of W1 are zero and the output
    layer starts small."""
    rng = np.random.default_rng(seed)
    p = np.zeros(PARAM_COUNT, np.float32)
    w1 = rng.normal(0, np.sqrt(2.0 / 14), (128, 16)).astype(np.float32)
    w1[:, 14:] = 0
    p[OFF_W1:OFF_B1] = w1.ravel()
    p[OFF_W2:OFF_B2] = rng.normal(0, np.sqrt(2.0 / 128), 128 * 128)
    p[OFF_W3:OFF_B3] = rng.normal(0, np.sqrt(2.0 / 128), 128 * 128)
    p[OFF_W4:OFF_B4] = rng.normal(0, 0.01, 3 * 128)
    return p


class Mlp:
    """The network on the GPU (axiom_mlp_*)."""

    def __init__(self, lib=None, device: int = -1, params: np.ndarray | None = None):
        self.lib = lib or ax.load_library()
        self._h = ctypes.c_void_p()
        ax._check(self.lib.axiom_mlp_create(device, ctypes.byref(self._h)), "axiom_mlp_create")
        self.set_params(init_params() if params is None else params)

    def close(self):
        if self._h:
            self.lib.axiom_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        ax._check(self.lib.axiom_mlp_set_params(self._h, ax._fptr(p), p.size), "axiom_mlp_set_params")

    def params(self) -> np.ndarray:
        p = np.empty(PARAM_COUNT, np.float32)
        ax._check(self.lib.axiom_mlp_get_params(self._h, ax._fptr(p), p.size), "axiom_mlp_get_params")
        return p

    def forward(self, feats: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(feats, np.float32)
        out = np.empty((len(f), 3), np.float32)
        ax._check(self.lib.axiom_mlp_forward(self._h, ax._fptr(f), len(f), ax._fptr(out)), "axiom_mlp_forward")
        return out

    def gradients(self, feats: np.ndarray, targets: np.ndarray) -> tuple[np.ndarray, float]:
        f = np.ascontiguousarray(feats, np.float32)
        t = np.ascontiguousarray(targets, np.float32)
        g = np.empty(PARAM_COUNT, np.float32)
        loss = ctypes.c_float()
        ax._check(self.lib.axiom_mlp_gradients(self._h, ax._fptr(f), ax._fptr(t), len(f), ax._fptr(g),
                                               ctypes.byref(loss)), "axiom_mlp_gradients")
        return g, float(loss.value)

    def train(self, feats, targets, epochs=1, batch=8192, lr=1e-3, seed=0) -> float:
        f = np.ascontiguousarray(feats, np.float32)
        t = np.ascontiguousarray(targets, np.float32)
        loss = ctypes.c_float()
        ax._check(self.lib.axiom_mlp_train(self._h, ax._fptr(f), ax._fptr(t), len(f), epochs, batch, lr, seed,
                                           ctypes.byref(loss)), "axiom_mlp_train")
        return float(loss.value)


@dataclass
class Standardizer:
    """Per-column affine maps used for training and folded into the exported weights."""
    f_mean: np.ndarray
    f_std: np.ndarray
    t_mean: np.ndarray
    t_std: np.ndarray

    @classmethod
    def fit(cls, f: np.ndarray, t: np.ndarray) -> "Standardizer":
        fs = f.std(0)
        ts = t.std(0)
        return cls(f.mean(0), np.where(fs > 1e-6, fs, 1.0), t.mean(0), np.where(ts > 1e-6, ts, 1.0))

    def features(self, f):
        return ((f - self.f_mean) / self.f_std).astype(np.float32)

    def targets(self, t):
        return ((t - self.t_mean) / self.t_std).astype(np.float32)

    def fold(self, p: np.ndarray) -> np.ndarray:
        """Parameters for raw features / raw targets from ones trained on standardized data:
        W1' = W1 / std, b1' = b1 - W1' mean; W4' = diag(t_std) W4, b4' = t_std b4 + t_mean."""
        q = p.astype(np.float64).copy()
        w1 = q[OFF_W1:OFF_B1].reshape(128, 16)
        w1n = w1.copy()
        w1n[:, :14] = w1[:, :14] / self.f_std
        q[OFF_B1:OFF_W2] = q[OFF_B1:OFF_W2] - w1n[:, :14] @ self.f_mean
        q[OFF_W1:OFF_B1] = w1n.ravel()
        w4 = q[OFF_W4:OFF_B4].reshape(3, 128) * self.t_std[:, None]
        q[OFF_W4:OFF_B4] = w4.ravel()
        q[OFF_B4:] = q[OFF_B4:] * self.t_std + self.t_mean
        return q.astype(np.float32)


def train_network(lib, f, t, epochs=20, batch=8192, lr=1e-3, decay=0.85, seed=0, log=None):
    """Trains on standardized data on the GPU; returns (raw-unit parameters, epoch losses)."""
    st = Standardizer.fit(f, t)
    fs, ts = st.features(f), st.targets(t)
    net = Mlp(lib, params=init_params(seed))
    losses = []
    for e in range(epochs):
        losses.append(net.train(fs, ts, epochs=1, batch=batch, lr=lr * decay ** e, seed=seed + e))
        if log:
            log(f"epoch {e}: loss {losses[-1]:.4f}")
    params = st.fold(net.params())
    net.close()
    return params, losses


def solver_config(lib, warm: int, dt: float = 1 / 60, tol: float = 1e-4, max_iter: int = 20000):
    return ax.default_config(lib, time_step=dt, residual_tolerance=tol, max_iterations=max_iter, warm_start=warm)


def generate_samples(lib, n_samples: int, towers: int = 256, seed: int = 1000, steps_per_scene: int = 60,
                     settle: int = 5, dt: float = 1 / 60, max_iter: int = 20000, log=None, params=None):
    """Solver samples (features, correction to the converged impulses) from seeded tower
    scenes: the plain solver's, or with `params` the solver warm-started by that network
    (the states the learned warm start visits, for a further training round)."""
    feats, targets = [], []
    total = 0
    s = seed
    while total < n_samples:
        scene = ax.Scene.towers(seed=s, count=towers, friction=0.6, lib=lib)
        warm = ax.WARM_PREVIOUS if params is None else ax.WARM_LEARNED
        w = ax.PhysicsWorld(solver_config(lib, warm, dt, max_iter=max_iter), lib=lib)
        w.add_bodies(scene.bodies)
        if params is not None:
            w.set_warm_start_model(params)
        w.set_recording(True)
        for k in range(steps_per_scene):
            w.step(dt, check=False)
            if k < settle:
                continue
            f, t, _ = w.read_samples()
            feats.append(f)
            targets.append(t)
            total += len(f)
            if total >= n_samples:
                break
        if log:
            log(f"scene seed {s}: {total} samples")
        w.close()
        s += 1
    f = np.concatenate(feats)[:n_samples]
    t = np.concatenate(targets)[:n_samples]
    return f, t


@dataclass
class EvalResult:
    iterations: list
    step_ms: list
    solver_ms: list
    residual: list

    def summary(self) -> dict:
        return {"mean_iterations": float(np.mean(self.iterations)), "iterations": list(map(int, self.iterations)),
                "mean_step_ms": float(np.mean(self.step_ms)),
                "mean_solver_ms": float(np.mean(self.solver_ms)),
                "max_residual": float(np.max(self.residual)), "steps": len(self.iterations)}


def evaluate(lib, params, towers: int = 256, seed: int = 11, steps: int = 8, settle: int = 5, dt: float = 1 / 60,
             max_iter: int = 20000) -> dict:
    """Iterations and time to the residual threshold, plain vs learned warm start.  The
    scene settles for `settle` steps under the plain solver; both arms then resume that
    same state (a snapshot, previous-step impulses included) and step `steps` steps."""
    scene = ax.Scene.towers(seed=seed, count=towers, friction=0.6, lib=lib)
    w = ax.PhysicsWorld(solver_config(lib, ax.WARM_PREVIOUS, dt, max_iter=max_iter), lib=lib)
    w.add_bodies(scene.bodies)
    for _ in range(settle):
        w.step(dt, check=False)
    start = bytearray(w.save_snapshot())
    w.close()
    out = {"bodies": scene.n}
    for name, warm in (("plain", ax.WARM_PREVIOUS), ("learned", ax.WARM_LEARNED)):
        snap = bytearray(start)
        ax.SnapshotHeader.from_buffer(snap).config.warm_start = warm
        a = ax.PhysicsWorld(solver_config(lib, warm, dt, max_iter=max_iter), lib=lib)
        a.load_snapshot(bytes(snap))
        if warm == ax.WARM_LEARNED:
            a.set_warm_start_model(params)
        r = EvalResult([], [], [], [])
        for _ in range(steps):
            st = a.step(dt, check=False)
            r.iterations.append(st.iterations)
            r.step_ms.append(st.total_step_time)
            r.solver_ms.append(st.solver_time)
            r.residual.append(st.residual)
        out[name] = r.summary()
        a.close()
    out["iteration_reduction"] = 1.0 - out["learned"]["mean_iterations"] / out["plain"]["mean_iterations"]
    out["time_reduction"] = 1.0 - out["learned"]["mean_solver_ms"] / out["plain"]["mean_solver_ms"]
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=5_000_000)
    ap.add_argument("--towers", type=int, default=2048)
    ap.add_argument("--gen-towers", type=int, default=512, help="towers per training scene")
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval-steps", type=int, default=30)
    ap.add_argument("--rounds", type=int, default=1,
                    help="training rounds; each round after the first adds --round-samples samples recorded "
                         "with the previous round's network as the warm start and retrains on all samples")
    ap.add_argument("--round-samples", type=int, default=1_000_000)
    ap.add_argument("--save", default="")
    ap.add_argument("--out", default="")
    ap.add_argument("--forward-rows", type=int, default=0,
                    help="only run the network: 3 forwards and 1 gradient pass on this many random rows "
                         "(a small case for profiling the GEMM kernels), then exit")
    a = ap.parse_args(argv)
    lib = ax.load_library()
    if a.forward_rows:
        rng = np.random.default_rng(0)
        f = rng.normal(0, 1, (a.forward_rows, 14)).astype(np.float32)
        t = rng.normal(0, 1, (a.forward_rows, 3)).astype(np.float32)
        net = Mlp(lib)
        for _ in range(3):
            net.forward(f)
        net.gradients(f, t)
        net.close()
        return 0
    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
    t0 = time.time()
    f, t = generate_samples(lib, a.samples, towers=a.gen_towers, seed=1000, log=log)
    t1 = time.time()
    params, losses = train_network(lib, f, t, epochs=a.epochs, batch=a.batch, lr=a.lr, log=log)
    for r in range(1, a.rounds):
        fr, tr = generate_samples(lib, a.round_samples, towers=a.gen_towers, seed=1000 + 1000 * r, log=log,
                                  params=params)
        f, t = np.concatenate([f, fr]), np.concatenate([t, tr])
        params, losses = train_network(lib, f, t, epochs=a.epochs, batch=a.batch, lr=a.lr, log=log)
    t2 = time.time()
    if a.save:
        np.save(a.save, params)
    ev = evaluate(lib, params, towers=a.towers, seed=1, steps=a.eval_steps)  # separately seeded scene
    res = {"samples": len(f), "rounds": a.rounds, "train_towers_per_scene": a.gen_towers, "eval_towers": a.towers,
           "gen_s": t1 - t0, "train_s": t2 - t1, "epoch_loss_standardized": losses, **ev}
    print(json.dumps(res))
    if a.out:
        Path(a.out).write_text(json.dumps(res, indent=1) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
