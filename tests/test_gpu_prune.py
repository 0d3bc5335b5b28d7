"""Learned candidate pruning on the GPU: features, tensor-core forward, training
kernels (gradients and Adam against the CPU oracle), and the trained network in
the detection loop with the exact path as referee: zero missed contacts, identical
assembly, fewer pairs per Newton iteration."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from oracle import mlp as M  # noqa: E402
from xkgpu import prune as P  # noqa: E402
from xkgpu import workloads as W  # noqa: E402
from xkgpu.engine import AssemblyEngine  # noqa: E402


def _engine(w, precision="fp64"):
    st = w.strand
    return AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=precision, **w.engine_kwargs())


def _random_batch(n, seed):
    """Feature rows in the ranges the geometry produces."""
    rng = np.random.default_rng(seed)
    X = np.zeros((n, M.F), np.float32)
    X[:, 0] = rng.uniform(0.5, 8.0, n)
    X[:, 1] = rng.uniform(0.0, 1.0, n)
    X[:, 2] = rng.uniform(1.0, 6.0, n)
    X[:, 3] = rng.integers(0, 4, n) / 3.0
    X[:, 4] = rng.integers(0, 2, n)
    X[:, 5] = rng.uniform(-2.0, 8.0, n)
    X[:, 6] = rng.integers(0, 2, n)
    return X


def _theta(seed):
    th = M.init_params(seed)
    th[np.arange(th.size) % 7 == 3] += 0.05  # non-zero biases
    return th


def test_features_match_oracle():
    import ctypes as C

    from xkgpu import _lib as L
    from xkgpu.device import ptr, stream_handle

    w = W.config_workload("strand37", seed=2)
    eng = _engine(w)
    u0 = torch.as_tensor(w.u, device="cuda")
    rng = np.random.default_rng(9)
    u1h = w.u + rng.normal(0.0, 2e-3 * w.meta["d"], w.u.shape) * np.tile([1, 1, 1, 0, 0, 0], w.strand.n_nodes)
    u1 = torch.as_tensor(u1h, device="cuda")
    eng.detect(u0)
    pr = P.PairPruner()
    cands, nc = eng.candidates(u1)
    L.call("xk_nodes_prepare", C.byref(eng.mesh.c), ptr(u1), ptr(u1), ptr(eng.node32), stream_handle(None))
    feat, hist = pr.features(eng.mesh, eng.node32, cands, nc, eng.pairs)
    got = feat[: M.F * nc].view(nc, M.F).cpu().numpy()
    # oracle
    c = cands[: 2 * nc].view(-1, 2).cpu().numpy().astype(np.int64)
    st = w.strand
    x = st.coords + u1h.reshape(-1, 6)[:, 0:3]
    conn = np.asarray(st.conn, np.int64)
    old = eng.pair_state()
    ko = old["ea"] * (1 << 32) + old["eb"]
    kc = c[:, 0] * (1 << 32) + c[:, 1]
    j = np.searchsorted(ko, kc)
    j = np.minimum(j, ko.size - 1)
    has = ko[j] == kc
    layer = np.asarray(w.engine_kwargs()["layer"], np.int64)
    r = np.broadcast_to(np.asarray(st.radii, float), (conn.shape[0],))
    exp = M.features(x[conn[c[:, 0], 0]], x[conn[c[:, 0], 1]], x[conn[c[:, 1], 0]], x[conn[c[:, 1], 1]],
                     r[c[:, 0]], r[c[:, 1]], layer[c[:, 0]], layer[c[:, 1]], np.where(has, old["gap"][j], 0.0), has)
    assert np.array_equal(got, exp)
    hist_exp = has & ((old["status"][j] != 0) | (old["p_n"][j] > 0) | (old["k_pen"][j] > 0)
                      | np.any(old["z_t"][j] != 0, axis=1))
    assert np.array_equal(hist[:nc].cpu().numpy().astype(bool), hist_exp)


@pytest.mark.parametrize("n", [1, 37, 4096 + 5, 128 * 152 * 4 * 2 + 77])
def test_forward_matches_oracle(n):
    th = _theta(1)
    X = _random_batch(n, 3)
    pr = P.PairPruner(th)
    feat = torch.as_tensor(X.ravel(), device="cuda")
    exp, _ = M.forward(th, X)
    mma = pr.logits(feat, n, backend="mma").cpu().numpy()       # mma.sync tensor cores
    tc5 = pr.logits(feat, n, backend="tcgen05").cpu().numpy()   # tcgen05, TMEM accumulators
    assert not pr.tcgen05_failed()
    _, lt = pr.train_forward(feat, n)                           # training kernel
    scale = max(1.0, float(np.max(np.abs(exp))))
    # float sums in another order round the odd activation that sits at a bfloat16 tie to the
    # neighbouring value: nearly every row agrees to float rounding, the rest by one bfloat16 step
    for got in (mma, tc5, lt.cpu().numpy()):
        d = np.abs(got - exp)
        assert np.mean(d > 1e-5 * scale) <= 0.01
        assert np.max(d) <= 2.0**-6 * scale


def test_tcgen05_forward_reuses_pruner_and_zero_rows():
    """Zero feature rows give the network's constant response; repeated calls agree bit for bit."""
    th = _theta(4)
    pr = P.PairPruner(th, backend="tcgen05")
    n = 1000
    X = _random_batch(n, 5)
    X[::3] = 0.0
    feat = torch.as_tensor(X.ravel(), device="cuda")
    a = pr.logits(feat, n).cpu().numpy()
    b = pr.logits(feat, n).cpu().numpy()
    assert not pr.tcgen05_failed()
    assert np.array_equal(a, b)
    assert np.all(a[::3] == a[0])
    exp, _ = M.forward(th, X)
    assert np.max(np.abs(a - exp)) <= 2.0**-6 * max(1.0, float(np.max(np.abs(exp))))


def test_gradient_and_adam_match_oracle():
    n = 3000
    th = _theta(2)
    X = _random_batch(n, 5)
    rng = np.random.default_rng(6)
    y = (rng.random(n) < 0.25).astype(np.float32)
    wts = np.where(y > 0, 3.0, 1.0).astype(np.float32)
    pr = P.PairPruner(th)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
    loss, grad, _ = pr.gradient(dev(X.ravel()), dev(y), dev(wts), n)
    le, ge = M.loss_and_grad(th, X, y.astype(np.float64), wts.astype(np.float64))
    assert abs(float(loss.item()) - le) <= 1e-5 * abs(le)
    g = grad.cpu().numpy()
    assert rel_err(g, ge) < 1e-4
    # Adam on the same gradient: bit-identical float32 arithmetic
    pr.adam(torch.as_tensor(ge.astype(np.float32), device="cuda"), 1e-3)
    th2, _, _ = M.adam_step(th, ge.astype(np.float32), np.zeros_like(th), np.zeros_like(th), 1, 1e-3)
    assert np.array_equal(pr.theta.cpu().numpy(), th2)
    assert np.array_equal(pr.theta_bf16.cpu().numpy().view(np.uint16),
                          (M.bf16(th2).view(np.uint32) >> 16).astype(np.uint16))


def _training_set(pr, names_seeds):
    feats, ys = [], []
    for name, seed in names_seeds:
        w = W.config_workload(name, seed=seed)
        eng = _engine(w)
        rng = np.random.default_rng(100 + seed)
        u0 = torch.as_tensor(w.u, device="cuda")
        du = rng.normal(0.0, 3e-3 * w.meta["d"], w.u.shape) * np.tile([1, 1, 1, 0, 0, 0], w.strand.n_nodes)
        u1 = torch.as_tensor(w.u + du, device="cuda")
        f, y, _ = P.candidate_samples(eng, u0, u1, pr)
        feats.append(f)
        ys.append(y)
    return torch.cat(feats), torch.cat(ys)


def test_trained_pruner_in_detection_loop():
    pr = P.PairPruner(seed=0)
    feat, y = _training_set(pr, [("strand7", s) for s in range(4)] + [("strand37", s) for s in range(3)])
    rep = pr.fit(feat, y, epochs=300, lr=3e-3)
    assert rep.recall == 1.0
    assert rep.loss_last < rep.loss_first
    # held-out strand: every detection verified exactly
    w = W.config_workload("strand91", seed=11)
    exact, pruned = _engine(w, "mixed"), _engine(w, "mixed")
    pruned.set_pruner(pr, verify_every=1)
    rng = np.random.default_rng(5)
    u = w.u.copy()
    mask = np.tile([1, 1, 1, 0, 0, 0], w.strand.n_nodes)
    for inc in range(3):
        ud = torch.as_tensor(u, device="cuda")
        se, sp_ = exact.detect(ud), pruned.detect(ud)
        assert se["candidates"] == sp_["candidates"]
        assert sp_["members"] == se["members"]
        u1 = torch.as_tensor(u + rng.normal(0.0, 5e-4 * w.meta["d"], u.shape) * mask, device="cuda")
        exact.assemble(u1, ud)
        pruned.assemble(u1, ud)
        assert rel_err(pruned.R.cpu().numpy(), exact.R.cpu().numpy()) < 1e-12
        ke, kp = exact.K_contact_csr(), pruned.K_contact_csr()
        assert abs(ke - kp).max() <= 1e-12 * abs(ke).max()
        u = u1.cpu().numpy()
    st = pruned.prune_stats
    assert st["verified"] == 3 and st["missed"] == 0
    # the gain: the pair table (narrowphase work per detection and per Newton iteration) shrinks
    assert pruned.pairs.n < 0.8 * exact.pairs.n
    assert st["kept"] < 0.8 * st["candidates"]
    print("pairs exact", exact.pairs.n, "pruned", pruned.pairs.n, "kept", st["kept"], "of", st["candidates"])
