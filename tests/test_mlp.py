"""The warm-start network: the oracle's backprop, the GPU kernels against the oracle, and
the learned warm start inside the step.

The GPU network runs hand-written tcgen05 GEMMs with BF16 operands and FP32 accumulation;
the oracle evaluates the same network in double, rounding to bf16 where the GPU rounds,
so the two differ only by accumulation order: forward outputs agree to 2e-3 relative
(max-norm), gradients to 2e-2 relative (norm) per parameter block.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import axiom_gb300 as ax
import warmstart as ws

BLOCKS = {"W1": (ws.OFF_W1, ws.OFF_B1), "b1": (ws.OFF_B1, ws.OFF_W2), "W2": (ws.OFF_W2, ws.OFF_B2),
          "b2": (ws.OFF_B2, ws.OFF_W3), "W3": (ws.OFF_W3, ws.OFF_B3), "b3": (ws.OFF_B3, ws.OFF_W4),
          "W4": (ws.OFF_W4, ws.OFF_B4), "b4": (ws.OFF_B4, ws.PARAM_COUNT)}


def bind_oracle(oracle):
    F = ctypes.POINTER(ctypes.c_float)
    D = ctypes.POINTER(ctypes.c_double)
    oracle.oracle_mlp_forward.argtypes = [F, F, ctypes.c_uint32, F]
    oracle.oracle_mlp_forward.restype = ctypes.c_int32
    oracle.oracle_mlp_gradients.argtypes = [F, F, F, ctypes.c_uint32, D, D]
    oracle.oracle_mlp_gradients.restype = ctypes.c_int32
    oracle.oracle_mlp_set_rounding.argtypes = [ctypes.c_int32]
    oracle.oracle_mlp_set_rounding.restype = None
    return oracle


def oracle_forward(oracle, p, f):
    out = np.empty((len(f), 3), np.float32)
    oracle.oracle_mlp_forward(ax._fptr(p), ax._fptr(np.ascontiguousarray(f, np.float32)), len(f), ax._fptr(out))
    return out


def oracle_grads(oracle, p, f, t):
    g = np.empty(ws.PARAM_COUNT, np.float64)
    loss = ctypes.c_double()
    oracle.oracle_mlp_gradients(ax._fptr(p), ax._fptr(np.ascontiguousarray(f, np.float32)),
                                ax._fptr(np.ascontiguousarray(t, np.float32)), len(f),
                                g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(loss))
    return g, loss.value


def sample_data(n, seed=0):
    rng = np.random.default_rng(seed)
    f = rng.normal(0, 1, (n, 14)).astype(np.float32)
    t = (0.5 * f[:, 9:12] + 0.1 * np.tanh(f[:, 0:3])).astype(np.float32)
    return f, t


def torch_grads(p, f, t):
    """Independent fp64 autodiff of the same network (no bf16 rounding)."""
    torch = pytest.importorskip("torch")
    P = torch.tensor(p.astype(np.float64), requires_grad=True)
    X = torch.zeros(len(f), 16, dtype=torch.float64)
    X[:, :14] = torch.tensor(f.astype(np.float64))
    W1 = P[ws.OFF_W1:ws.OFF_B1].view(128, 16)
    W2 = P[ws.OFF_W2:ws.OFF_B2].view(128, 128)
    W3 = P[ws.OFF_W3:ws.OFF_B3].view(128, 128)
    W4 = P[ws.OFF_W4:ws.OFF_B4].view(3, 128)
    silu = torch.nn.functional.silu
    h = silu(X @ W1.T + P[ws.OFF_B1:ws.OFF_W2])
    h = silu(h @ W2.T + P[ws.OFF_B2:ws.OFF_W3])
    h = silu(h @ W3.T + P[ws.OFF_B3:ws.OFF_W4])
    y = h @ W4.T + P[ws.OFF_B4:]
    loss = ((y - torch.tensor(t.astype(np.float64))) ** 2).mean()
    loss.backward()
    return P.grad.numpy(), float(loss)


def test_oracle_backprop_matches_autodiff(oracle):
    o = bind_oracle(oracle)
    p = ws.init_params(3)
    p[ws.OFF_W4:ws.OFF_B4] = np.random.default_rng(1).normal(0, 0.2, 384)  # non-trivial head
    f, t = sample_data(64, 1)
    o.oracle_mlp_set_rounding(0)
    try:
        g, loss = oracle_grads(o, p, f, t)
    finally:
        o.oracle_mlp_set_rounding(1)
    gt, losst = torch_grads(p, f, t)
    assert abs(loss - losst) < 1e-5 * max(1.0, losst)
    for name, (a, b) in BLOCKS.items():
        ref = gt[a:b]
        err = np.linalg.norm(g[a:b] - ref) / max(np.linalg.norm(ref), 1e-12)
        assert err < 1e-4, (name, err)


def test_standardizer_fold_is_exact(oracle):
    """A network trained on standardized data, folded into raw units, computes the same
    function on raw inputs (checked in the oracle without bf16 rounding)."""
    o = bind_oracle(oracle)
    rng = np.random.default_rng(4)
    f = (rng.normal(0, 1, (256, 14)) * rng.uniform(0.1, 50, 14) + rng.normal(0, 5, 14)).astype(np.float32)
    t = (rng.normal(0, 1, (256, 3)) * [3.0, 0.5, 0.2] + [1.0, 0.0, -0.5]).astype(np.float32)
    st = ws.Standardizer.fit(f, t)
    p = ws.init_params(6)
    p[ws.OFF_W4:ws.OFF_B4] = rng.normal(0, 0.3, 384)
    o.oracle_mlp_set_rounding(0)
    try:
        y_std = oracle_forward(o, p, st.features(f)) * st.t_std + st.t_mean
        y_raw = oracle_forward(o, st.fold(p), f)
    finally:
        o.oracle_mlp_set_rounding(1)
    assert np.abs(y_std - y_raw).max() <= 1e-3 * max(1.0, np.abs(y_std).max())


@pytest.mark.gpu
def test_gpu_forward_matches_oracle(gpu_lib, oracle):
    o = bind_oracle(oracle)
    p = ws.init_params(5)
    p[ws.OFF_W4:ws.OFF_B4] = np.random.default_rng(2).normal(0, 0.2, 384)
    net = ws.Mlp(gpu_lib, params=p)
    for n in (1, 127, 128, 1000):
        f, _ = sample_data(n, n)
        yg = net.forward(f)
        yo = oracle_forward(o, p, f)
        err = np.abs(yg - yo).max() / max(np.abs(yo).max(), 1e-6)
        assert err < 2e-3, (n, err)


@pytest.mark.gpu
def test_gpu_gradients_match_oracle(gpu_lib, oracle):
    o = bind_oracle(oracle)
    p = ws.init_params(7)
    p[ws.OFF_W4:ws.OFF_B4] = np.random.default_rng(3).normal(0, 0.2, 384)
    net = ws.Mlp(gpu_lib, params=p)
    f, t = sample_data(1000, 4)
    gg, lg = net.gradients(f, t)
    go, lo = oracle_grads(o, p, f, t)
    assert abs(lg - lo) < 1e-3 * max(1.0, lo)
    for name, (a, b) in BLOCKS.items():
        ref = go[a:b]
        err = np.linalg.norm(gg[a:b] - ref) / max(np.linalg.norm(ref), 1e-12)
        assert err < 2e-2, (name, err)


@pytest.mark.gpu
def test_gpu_training_reduces_loss(gpu_lib):
    net = ws.Mlp(gpu_lib, params=ws.init_params(9))
    f, t = sample_data(16384, 5)
    _, l0 = net.gradients(f, t)
    for e in range(8):
        net.train(f, t, epochs=1, batch=1024, lr=2e-3, seed=e)
    _, l1 = net.gradients(f, t)
    assert l1 < 0.1 * l0, (l0, l1)


@pytest.mark.gpu
def test_gpu_training_is_reproducible(gpu_lib):
    """Gradients are summed in a fixed order (split and head-block partials), so the same
    seed and data give bit-identical weights, and two gradient calls agree bit for bit."""
    f, t = sample_data(8192, 6)
    runs = []
    for _ in range(2):
        net = ws.Mlp(gpu_lib, params=ws.init_params(11))
        g0, l0 = net.gradients(f, t)
        net.train(f, t, epochs=2, batch=2048, lr=1e-3, seed=3)
        runs.append((g0, l0, net.params()))
        net.close()
    (ga, la, pa), (gb, lb, pb) = runs
    assert np.array_equal(ga, gb) and la == lb
    assert np.array_equal(pa, pb)


@pytest.mark.gpu
def test_features_match_oracle(gpu_lib, oracle):
    """Recorded features and impulses of the GPU step equal the oracle's (same fp32 order)."""
    sc = ax.Scene.towers(seed=5, count=6, lib=gpu_lib)
    cfg = dict(time_step=1 / 60, velocity_iterations=10)
    g = ax.PhysicsWorld(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    w = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    for x in (g, w):
        x.add_bodies(sc.bodies)
        x.set_recording(True)
    for _ in range(6):
        g.step(1 / 60)
        w.step(1 / 60)
    fg, tg, kg = g.read_samples()
    fo, to, ko = w.read_samples()
    order_g = np.lexsort((kg[:, 2], kg[:, 1], kg[:, 0]))
    order_o = np.lexsort((ko[:, 2], ko[:, 1], ko[:, 0]))
    assert np.array_equal(kg[order_g], ko[order_o])
    assert np.array_equal(fg[order_g], fo[order_o])
    assert np.array_equal(tg[order_g], to[order_o])
    assert np.abs(fg[:, 9:12]).max() > 0  # previous impulses are present after step 1


@pytest.mark.gpu
def test_learned_warm_start_step_matches_oracle(gpu_lib, oracle):
    """With the same network both sides start PGS from nearly the same impulses (GPU
    bf16 GEMMs vs oracle) and iterate to the same threshold."""
    sc = ax.Scene.towers(seed=8, count=6, lib=gpu_lib)
    p = ws.init_params(11)
    p[ws.OFF_B4] = 1.0  # a non-zero normal impulse prediction
    cfg = dict(time_step=1 / 60, residual_tolerance=1e-4, max_iterations=3000, warm_start=ax.WARM_LEARNED)
    g = ax.PhysicsWorld(ax.default_config(gpu_lib, **cfg), lib=gpu_lib)
    w = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
    for x in (g, w):
        x.add_bodies(sc.bodies)
        x.set_warm_start_model(p)
    sg = g.step(1 / 60, check=False)
    so = w.step(1 / 60, check=False)
    assert sg.manifold_count == so.manifold_count and sg.colour_count == so.colour_count
    cg = ax.canonical_contacts(g.read_contacts())
    co = ax.canonical_contacts(w.read_contacts())
    scale = np.abs(co["impulse"]).max()
    assert np.abs(cg["impulse"] - co["impulse"]).max() <= 2e-3 * scale
    assert abs(sg.iterations - so.iterations) <= max(5, 0.05 * so.iterations)
