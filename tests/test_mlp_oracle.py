"""The pruning-MLP oracle on the CPU: its backward against finite differences, its
bfloat16 rounding against torch's, and the shared parameter initialisation."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import mlp as M

torch = pytest.importorskip("torch")


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    th = M.init_params(3).astype(np.float64)
    X = rng.normal(size=(60, M.F))
    y = (rng.random(60) < 0.3).astype(float)
    w = 1.0 + rng.random(60)
    _, g = M.loss_and_grad(th, X, y, w, quantize=False)
    idx = rng.choice(M.N_PARAMS, 60, replace=False)
    fd = np.empty(idx.size)
    for n, i in enumerate(idx):
        e = np.zeros_like(th)
        e[i] = 1e-6
        lp = M.loss_and_grad(th + e, X, y, w, quantize=False)[0]
        lm = M.loss_and_grad(th - e, X, y, w, quantize=False)[0]
        fd[n] = (lp - lm) / 2e-6
    assert np.max(np.abs(fd - g[idx])) <= 1e-7 * np.max(np.abs(g[idx]))


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.normal(size=2000) * 10.0 ** rng.integers(-30, 30, 2000),
                        np.array([0.0, -0.0, 1.0, 1.00390625, 1.01171875, 3.0e38, -3.3e38, 1e-40, -1e-41])])
    x = x.astype(np.float32)
    ref = torch.tensor(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(M.bf16(x), ref)


def test_quantized_forward_rounds_activations():
    th = M.init_params(0)
    X = np.random.default_rng(4).normal(size=(10, M.F)).astype(np.float32)
    _, c = M.forward(th, X)
    for k in ("x0", "a1", "a2", "a3"):
        assert np.array_equal(c[k], M.bf16(c[k]))


def test_product_init_matches_oracle():
    from xkgpu import prune as P

    assert np.array_equal(P.init_params(7), M.init_params(7))
    assert P.NPARAM == M.N_PARAMS
