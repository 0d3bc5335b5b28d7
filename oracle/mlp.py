"""CPU oracle of the pair-pruning MLP (test infrastructure only).

The reference has no learned component; this file is the specification the GPU
kernels are checked against.  Network: F = 8 inputs -> 64 -> 64 -> 64 -> 1,
ReLU between layers, sigmoid output.  The forward pass rounds the weights, the
inputs and every hidden activation to bfloat16 (round to nearest even) and
accumulates in float32, as the GPU does; the backward pass is plain float32
(no rounding of gradients); the ReLU derivative is taken where the (rounded)
activation is positive.

Parameters are one flat float32 vector in this order:
W1 (64 x F, row-major), b1 (64), W2 (64 x 64), b2 (64), W3 (64 x 64), b3 (64), w4 (64), b4 (1).
"""

from __future__ import annotations

import numpy as np

F, H = 8, 64
SIZES = [("W1", (H, F)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
         ("w4", (H,)), ("b4", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(theta: np.ndarray) -> dict:
    out, o = {}, 0
    for k, s in SIZES:
        n = int(np.prod(s))
        out[k] = theta[o:o + n].reshape(s)
        o += n
    return out


def bf16(x) -> np.ndarray:
    """Round float32 to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    nan = np.isnan(a)
    if nan.any():
        out = out.copy()
        out[nan] = np.nan
    return out


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights, zero biases (float32 master copy)."""
    rng = np.random.default_rng(seed)
    parts = []
    for k, s in SIZES:
        if k.startswith("b"):
            parts.append(np.zeros(s, np.float32))
        else:
            fan_in = s[-1] if len(s) == 2 else H
            parts.append((rng.normal(size=s) * np.sqrt(2.0 / fan_in)).astype(np.float32))
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


def forward(theta: np.ndarray, X: np.ndarray, *, quantize: bool = True):
    """Scores (logits) and the cached activations of a batch X (n x F).

    quantize=False runs the same network unrounded in float64 (used to pin the
    backward pass against finite differences).
    """
    if quantize:
        q, dt = bf16, np.float32
    else:
        def q(a):
            return np.asarray(a, np.float64)
        dt = np.float64
    p = {k: q(v) for k, v in unpack(np.asarray(theta, dt)).items()}
    x0 = q(X)
    z1 = x0 @ p["W1"].T + p["b1"]
    a1 = q(np.maximum(z1, 0.0))
    z2 = a1 @ p["W2"].T + p["b2"]
    a2 = q(np.maximum(z2, 0.0))
    z3 = a2 @ p["W3"].T + p["b3"]
    a3 = q(np.maximum(z3, 0.0))
    logit = a3 @ p["w4"] + p["b4"][0]
    return logit.astype(dt), dict(x0=x0, a1=a1, a2=a2, a3=a3, z1=z1, z2=z2, z3=z3, p=p)


def loss_and_grad(theta: np.ndarray, X: np.ndarray, y: np.ndarray, w: np.ndarray, *, quantize: bool = True):
    """Weighted mean binary cross-entropy on the logits and its gradient (flat).

    loss = sum_i w_i * (softplus(l_i) - y_i l_i) / n; d loss / d l_i = w_i (sigmoid(l_i) - y_i) / n.
    With quantize=True the gradient passes through the bfloat16 rounding as the
    identity (the rounded activations and weights are used in the chain rule).
    """
    dt = np.float32 if quantize else np.float64
    n = X.shape[0]
    logit, c = forward(theta, X, quantize=quantize)
    p = c["p"]
    lf = logit.astype(np.float64)
    loss = float(np.sum(w * (np.logaddexp(0.0, lf) - y * lf)) / n)
    g = (w * (1.0 / (1.0 + np.exp(-lf)) - y) / n).astype(dt)
    grads = {"w4": c["a3"].T @ g, "b4": np.array([g.sum()], dt)}
    d3 = np.outer(g, p["w4"]) * (c["a3"] > 0)
    grads["W3"], grads["b3"] = d3.T @ c["a2"], d3.sum(0)
    d2 = (d3 @ p["W3"]) * (c["a2"] > 0)
    grads["W2"], grads["b2"] = d2.T @ c["a1"], d2.sum(0)
    d1 = (d2 @ p["W2"]) * (c["a1"] > 0)
    grads["W1"], grads["b1"] = d1.T @ c["x0"], d1.sum(0)
    flat = np.concatenate([np.asarray(grads[k], dt).ravel() for k, _ in SIZES])
    return loss, flat


def adam_step(theta, grad, m, v, step: int, lr: float, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (bias-corrected), float32, returns the new (theta, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1**step)
    vh = v / (1 - b2**step)
    return (theta - lr * mh / (np.sqrt(vh) + eps)).astype(np.float32), m.astype(np.float32), v.astype(np.float32)


def split(x):
    """Positions as float hi/lo pairs, as the node records hold them (``xk_nodes_prepare``):
    hi = float(x), lo = float(x - hi)."""
    x = np.asarray(x, dtype=np.float64)
    hi = x.astype(np.float32)
    return hi, (x - hi.astype(np.float64)).astype(np.float32)


def split_diff(p, q):
    """p - q of two split positions: (p_hi - q_hi) + (p_lo - q_lo), each float32 operation rounded."""
    return (p[0] - q[0]) + (p[1] - q[1])


def current_gap_f(A, B, Wv, rs):
    """(segment distance - rs) / rs in float32 from the float32 segment differences A = a1 - a0,
    B = b1 - b0, Wv = a0 - b0: the clamped closest point of ``_closest_point_segments_batch``
    (``geometry/_compute.py:55-151``) in float32 with every operation rounded on its own; near-parallel
    pairs (det <= 1e-3 ac) take s = 0."""
    f = np.float32

    def dot(p, q):
        return (p[:, 0] * q[:, 0] + p[:, 1] * q[:, 1]) + p[:, 2] * q[:, 2]

    a, b, c, d, e = dot(A, A), dot(A, B), dot(B, B), dot(A, Wv), dot(B, Wv)
    ac = a * c
    det = ac - b * b
    par = ~(det > f(1e-3) * ac)
    with np.errstate(invalid="ignore", divide="ignore"):
        sdet = np.where(par, f(1.0), det)
        su, tu = (b * e - c * d) / sdet, (a * e - b * d) / sdet
        cl = lambda v: np.clip(v, f(0.0), f(1.0))  # noqa: E731
        csafe, asafe = np.where(c > 0, c, f(1.0)), np.where(a > 0, a, f(1.0))
        s = np.where(par, f(0.0), cl(su))
        t = np.where(par, np.where(c > 0, cl(e / csafe), f(0.0)), cl(tu))
        s_cl = ~par & ((su < 0) | (su > 1))
        t = np.where(s_cl, np.where(c > 0, cl((b * s + e) / csafe), f(0.0)), t)
        t_cl = ~par & ((tu < 0) | (tu > 1))
        s = np.where(t_cl, np.where(a > 0, cl((b * t - d) / asafe), f(0.0)), s)
        t = np.where(t_cl, np.where(c > 0, cl((b * s + e) / csafe), f(0.0)), t)
    D = (Wv + s[:, None] * A) - t[:, None] * B
    rsf = np.asarray(rs, dtype=np.float64).astype(f)
    return ((np.sqrt(dot(D, D)) - rsf) / rsf).astype(np.float64)


def features(xa0, xa1, xb0, xb1, ra, rb, la, lb, prev_gap, has_prev):
    """Per-candidate inputs (n x F), float32.  The positions (X + u, double) are split into float hi/lo
    pairs as the node records hold them; the differences are taken from the pairs and everything after
    them in float32 with every operation rounded on its own (the GPU kernel's order).

    0: |m_a - m_b| / (r_a + r_b)              midpoint separation
    1: |d_a . d_b| / (|d_a| |d_b|)            cosine of the tangent angle
    2: (|d_a| + |d_b|) / (2 (r_a + r_b))      half lengths
    3: min(|layer_a - layer_b|, 3) / 3        layer distance (0 without layers)
    4: 1 if either layer is 0 (the core)
    5: previous-step gap / (r_a + r_b), clipped to [-2, 8]; without one, the
       current gap (segment distance - r_a - r_b) / (r_a + r_b) in float
       (``current_gap_f``)
    6: 1 if the previous-step gap exists
    7: 0
    """
    f = np.float32
    rs = ra + rb
    rsf = np.asarray(rs, dtype=np.float64).astype(f)
    a0, a1, b0, b1 = split(xa0), split(xa1), split(xb0), split(xb1)
    da, db, dw = split_diff(a1, a0), split_diff(b1, b0), split_diff(a0, b0)
    dm = f(0.5) * (dw + split_diff(a1, b1))

    def dot(p, q):
        return (p[:, 0] * q[:, 0] + p[:, 1] * q[:, 1]) + p[:, 2] * q[:, 2]

    with np.errstate(invalid="ignore", divide="ignore"):
        sep = np.sqrt(dot(dm, dm))
        la_n, lb_n = np.sqrt(dot(da, da)), np.sqrt(dot(db, db))
        den = la_n * lb_n
        den = np.where((den >= f(1e-30)) | np.isnan(den), den, f(1e-30))
        X = np.zeros((xa0.shape[0], F), np.float32)
        X[:, 0] = sep / rsf
        X[:, 1] = np.abs(dot(da, db)) / den
        X[:, 2] = (la_n + lb_n) / (f(2.0) * rsf)
        have_layer = (la >= 0) & (lb >= 0)
        X[:, 3] = np.where(have_layer, np.minimum(np.abs(la - lb), 3).astype(f) / f(3.0), f(0.0))
        X[:, 4] = np.where(have_layer & ((la == 0) | (lb == 0)), f(1.0), f(0.0))
        prev = np.asarray(prev_gap, dtype=np.float64).astype(f) / rsf
        X[:, 5] = np.clip(np.where(has_prev, prev, current_gap_f(da, db, dw, rs).astype(f)), f(-2.0), f(8.0))
        X[:, 6] = has_prev.astype(np.float32)
    return X
