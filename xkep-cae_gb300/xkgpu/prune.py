"""Learned pruning of broadphase candidate pairs.

A BF16 MLP (8 -> 64 -> 64 -> 64 -> 1) scores every broadphase candidate from
cheap geometric features; candidates scored below a threshold stay out of the
pair table, so the per-iteration narrowphase and the detection narrowphase run
on fewer pairs.  Pairs with contact history are never pruned, and the exact
broadphase + narrowphase remains the referee: ``AssemblyEngine`` checks the
pruned candidates exactly every ``verify_every`` detections and puts back any
that the exact path would activate.

The network is trained on the GPU by the xkgpu kernels (forward with stored
activations, backward, fixed-order weight-gradient reduction, Adam) on labels
produced by the exact narrowphase itself: a candidate is positive when its gap
is at most ``label_margin * (r_a + r_b)`` (0.1 by default: candidates farther
apart than a tenth of the radius sum are the ones to drop).  The threshold is set below the
smallest positive score of the training set, so every training positive is
kept.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L
from .device import DeviceMesh, DevicePairTable, ptr, require_cuda, stream_handle

F, H, NPARAM = L.MLP_IN, L.MLP_HIDDEN, L.MLP_PARAMS
_LAYOUT = [("W1", (H, F)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
           ("w4", (H,)), ("b4", (1,))]


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights, zero biases, in the flat parameter layout of the kernels."""
    rng = np.random.default_rng(seed)
    parts = []
    for k, s in _LAYOUT:
        if k.startswith("b"):
            parts.append(np.zeros(int(np.prod(s)), np.float32))
        else:
            fan_in = s[-1] if len(s) == 2 else H
            parts.append((rng.normal(size=s) * np.sqrt(2.0 / fan_in)).astype(np.float32).ravel())
    out = np.concatenate(parts)
    assert out.size == NPARAM
    return out


@dataclass
class TrainReport:
    epochs: int
    loss_first: float
    loss_last: float
    n_samples: int
    n_positive: int
    threshold: float
    recall: float
    kept_fraction: float


class PairPruner:
    """The pruning network: parameters on the device, training and scoring through the C ABI."""

    def __init__(self, theta: np.ndarray | None = None, *, threshold: float = -np.inf, label_margin: float = 0.1,
                 seed: int = 0, device=None, backend: str = "tcgen05"):
        self.device = require_cuda(device)
        th = init_params(seed) if theta is None else np.asarray(theta, np.float32)
        if th.size != NPARAM:
            raise ValueError(f"expected {NPARAM} parameters, got {th.size}")
        self.theta = torch.as_tensor(th.copy(), device=self.device)
        self.theta_bf16 = torch.zeros(NPARAM, dtype=torch.int16, device=self.device)
        self._m = torch.zeros(NPARAM, dtype=torch.float32, device=self.device)
        self._v = torch.zeros(NPARAM, dtype=torch.float32, device=self.device)
        self.step = 0
        self.threshold = float(threshold)
        self.label_margin = float(label_margin)
        self.backend = backend
        self._tc_err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.sync_bf16()

    # ------------------------------------------------------------------ parameters
    def sync_bf16(self, stream=None):
        L.call("xk_mlp_to_bf16", ptr(self.theta), ptr(self.theta_bf16), stream_handle(stream))

    def state_dict(self) -> dict:
        return {"theta": self.theta.cpu().numpy().copy(), "threshold": np.float64(self.threshold),
                "label_margin": np.float64(self.label_margin)}

    @classmethod
    def from_state(cls, d: dict, device=None) -> "PairPruner":
        return cls(np.asarray(d["theta"], np.float32), threshold=float(d["threshold"]),
                   label_margin=float(d["label_margin"]), device=device)

    # ------------------------------------------------------------------ kernels
    def features(self, mesh: DeviceMesh, node32: torch.Tensor, cands: torch.Tensor, n: int,
                 old: DevicePairTable, stream=None):
        """(feat [n x 8] float, hist [n] uint8) of candidate rows cands[:n] at the positions of the node
        records ``node32`` (``xk_nodes_prepare``)."""
        feat = torch.empty(max(n, 1) * F, dtype=torch.float32, device=self.device)
        hist = torch.empty(max(n, 1), dtype=torch.uint8, device=self.device)
        L.call("xk_prune_features", C.byref(mesh.c), ptr(node32), ptr(cands), int(n), C.byref(old.c), ptr(feat),
               ptr(hist), stream_handle(stream))
        return feat, hist

    def logits(self, feat: torch.Tensor, n: int, stream=None, backend: str | None = None) -> torch.Tensor:
        """Scores of n samples.  backend "mma" (mma.sync) or "tcgen05" (TMEM
        accumulators); default: the pruner's ``backend`` attribute."""
        out = torch.empty(max(n, 1), dtype=torch.float32, device=self.device)
        b = backend or self.backend
        if b == "tcgen05":
            self._tc_err.zero_()
            L.call("xk_mlp_forward_tcgen05", ptr(self.theta_bf16), ptr(feat), int(n), ptr(out), ptr(self._tc_err),
                   stream_handle(stream))
        elif b == "mma":
            L.call("xk_mlp_forward", ptr(self.theta_bf16), ptr(feat), int(n), ptr(out), stream_handle(stream))
        else:
            raise ValueError(f"unknown backend {b!r}")
        return out[:n]

    def tcgen05_failed(self) -> bool:
        """True if the last tcgen05 scoring hit an expired completion wait (synchronises)."""
        return bool(self._tc_err.item())

    def train_forward(self, feat: torch.Tensor, n: int, stream=None):
        act = torch.empty(L.MLP_ACT * n, dtype=torch.float32, device=self.device)
        logit = torch.empty(n, dtype=torch.float32, device=self.device)
        L.call("xk_mlp_train_forward", ptr(self.theta), ptr(feat), int(n), ptr(act), ptr(logit),
               stream_handle(stream))
        return act, logit

    def gradient(self, feat, y, w, n: int, stream=None):
        """(loss, grad) of the weighted mean BCE over n samples; both on the device."""
        act, logit = self.train_forward(feat, n, stream)
        dvec = torch.empty(L.MLP_ACT * n, dtype=torch.float32, device=self.device)
        g = torch.empty(n, dtype=torch.float32, device=self.device)
        grad = torch.empty(NPARAM, dtype=torch.float32, device=self.device)
        loss = torch.empty(1, dtype=torch.float32, device=self.device)
        L.call("xk_mlp_backward", ptr(self.theta), ptr(feat), ptr(act), ptr(logit), ptr(y), ptr(w), int(n),
               ptr(dvec), ptr(g), ptr(grad), ptr(loss), stream_handle(stream))
        return loss, grad, logit

    def adam(self, grad, lr: float, stream=None, b1=0.9, b2=0.999, eps=1e-8):
        self.step += 1
        L.call("xk_mlp_adam", ptr(self.theta), ptr(grad), ptr(self._m), ptr(self._v), self.step, float(lr),
               float(b1), float(b2), float(eps), ptr(self.theta_bf16), stream_handle(stream))

    # ------------------------------------------------------------------ training
    def fit(self, feat: torch.Tensor, y: torch.Tensor, *, epochs: int = 400, lr: float = 3e-3,
            pos_weight: float | None = None, threshold_margin: float = 1.0) -> TrainReport:
        """Full-batch Adam on (feat, y), then the recall-1 threshold on the training set."""
        n = int(y.numel())
        yf = y.to(torch.float32)
        npos = int(yf.sum().item())
        if pos_weight is None:
            pos_weight = max(1.0, (n - npos) / max(npos, 1))
        w = torch.where(yf > 0.5, torch.full_like(yf, float(pos_weight)), torch.ones_like(yf))
        first = last = float("nan")
        for e in range(epochs):
            loss, grad, _ = self.gradient(feat, yf, w, n)
            self.adam(grad, lr)
            if e == 0:
                first = float(loss.item())
        loss, _, _ = self.gradient(feat, yf, w, n)
        last = float(loss.item())
        logit = self.logits(feat, n)
        pos = logit[yf > 0.5]
        self.threshold = float(pos.min().item()) - threshold_margin if npos else float("inf")
        kept = float((logit >= self.threshold).float().mean().item())
        recall = float((pos >= self.threshold).float().mean().item()) if npos else 1.0
        return TrainReport(epochs, first, last, n, npos, self.threshold, recall, kept)


# ---------------------------------------------------------------------- training data


def candidate_samples(engine, u0: torch.Tensor, u1: torch.Tensor, pruner: PairPruner):
    """Features and exact labels of the candidates at u1, with the table detected at u0 as history.

    Runs the exact path of ``engine`` (an ``AssemblyEngine``): detection at u0,
    the broadphase at u1, the features against the u0 table, then the exact
    detection at u1 whose narrowphase gaps give the labels.
    """
    engine.detect(u0)
    cands, nc = engine.candidates(u1)
    L.call("xk_nodes_prepare", C.byref(engine.mesh.c), ptr(u1), ptr(u1), ptr(engine.node32), stream_handle(None))
    feat, _ = pruner.features(engine.mesh, engine.node32, cands, nc, engine.pairs)
    engine.detect(u1)
    h = engine.pairs
    n = h.n
    key_t = h.t["ea"][:n].to(torch.int64) * (1 << 32) + h.t["eb"][:n].to(torch.int64)
    c = cands[: 2 * nc].view(-1, 2).to(torch.int64)
    key_c = c[:, 0] * (1 << 32) + c[:, 1]
    idx = torch.searchsorted(key_t, key_c)
    gap = h.t["gap"][:n][idx]
    rs = engine.mesh.radii[c[:, 0]] + engine.mesh.radii[c[:, 1]]
    y = (gap <= pruner.label_margin * rs).to(torch.float32)
    return feat[: F * nc].clone(), y, nc
