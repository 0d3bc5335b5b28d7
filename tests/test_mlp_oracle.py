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


def test_features_from_split_positions_agree_with_double_differences():
    """The features take their position differences from the float hi/lo pairs of the node records; they
    agree with differences taken in double and rounded once to within float rounding of each feature."""
    rng = np.random.default_rng(4)
    n = 5000
    centre = rng.uniform(-20.0, 20.0, (n, 3))  # coordinates in mm, strand scale
    xa0 = centre + rng.normal(0.0, 0.5, (n, 3))
    xa1 = xa0 + rng.normal(0.0, 0.5, (n, 3))
    xb0 = centre + rng.normal(0.0, 0.6, (n, 3))
    xb1 = xb0 + rng.normal(0.0, 0.5, (n, 3))
    ra, rb = np.full(n, 0.25), np.full(n, 0.25)
    la, lb = rng.integers(0, 5, n), rng.integers(0, 5, n)
    has = rng.random(n) < 0.5
    prev = rng.normal(0.0, 0.3, n)
    X = M.features(xa0, xa1, xb0, xb1, ra, rb, la, lb, prev, has)
    # the same features from differences taken in double
    f = np.float32
    rs = (ra + rb).astype(f)
    dm = (0.5 * (xa0 + xa1) - 0.5 * (xb0 + xb1)).astype(f)
    da, db = (xa1 - xa0).astype(f), (xb1 - xb0).astype(f)
    nrm = lambda v: np.sqrt(np.sum(v.astype(np.float64) ** 2, axis=1))  # noqa: E731
    ref0 = nrm(dm) / rs
    ref1 = np.abs(np.sum(da.astype(np.float64) * db, axis=1)) / (nrm(da) * nrm(db))
    ref2 = (nrm(da) + nrm(db)) / (2.0 * rs)
    for got, ref in ((X[:, 0], ref0), (X[:, 1], ref1), (X[:, 2], ref2)):
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)) < 1e-5
    # the previous gap where it exists, and the split of a position recomposes it to double accuracy
    assert np.array_equal(X[has, 5], np.clip((prev[has].astype(f) / rs[has]), -2.0, 8.0).astype(f))
    hi, lo = M.split(xa0)
    assert np.max(np.abs((hi.astype(np.float64) + lo) - xa0)) <= 2.0 ** -46 * np.max(np.abs(xa0))
