"""Batched strands: many independent strands, each with its own friction
coefficient, assembled by the same launches as one mesh.  Every instance's
residual, contact tangent and pair states equal those of a separate engine
built on that instance alone."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from xkgpu import workloads as W  # noqa: E402
from xkgpu.engine import AssemblyEngine  # noqa: E402


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_separate_instances(precision):
    w = W.config_workload("batch8", seed=3)
    st = w.strand
    inst, first = w.meta["instance"], w.meta["node_first"]
    mus = w.meta["mu_instance"]
    assert len(set(np.round(mus, 6))) > 1  # the instances really differ in mu
    batch = AssemblyEngine(st.coords, st.conn, st.radii, w.section, layer=st.elem_layer, precision=precision,
                           k_pen=w.k_pen, mu=w.mu)
    u = torch.as_tensor(w.u, device="cuda")
    rng = np.random.default_rng(1)
    du = rng.normal(0.0, 2e-3 * w.meta["d"], w.u.shape) * np.tile([1, 1, 1, 0, 0, 0], st.n_nodes)
    u1 = torch.as_tensor(w.u + du, device="cuda")
    sb = batch.detect(u)
    batch.assemble(u1, u)
    Rb = batch.R.cpu().numpy()
    Kb = batch.K_contact_csr()
    hb = batch.pair_state()
    n_nodes_all = st.n_nodes
    bounds = list(first) + [n_nodes_all]
    pairs_total = 0
    for k in range(len(first)):
        n0, n1 = int(bounds[k]), int(bounds[k + 1])
        el = np.nonzero(inst == k)[0]
        e0, e1 = int(el[0]), int(el[-1]) + 1
        eng = AssemblyEngine(st.coords[n0:n1], st.conn[e0:e1] - n0, st.radii[e0:e1], w.section,
                             layer=st.elem_layer[e0:e1], precision=precision, k_pen=w.k_pen, mu=float(mus[k]))
        uk = torch.as_tensor(w.u[6 * n0:6 * n1], device="cuda")
        u1k = torch.as_tensor((w.u + du)[6 * n0:6 * n1], device="cuda")
        eng.detect(uk)
        eng.assemble(u1k, uk)
        pairs_total += eng.pairs.n
        Rk = eng.R.cpu().numpy()
        assert rel_err(Rb[6 * n0:6 * n1], Rk) < 1e-12, k
        Kk = eng.K_contact_csr()
        Kbk = Kb[6 * n0:6 * n1, 6 * n0:6 * n1]
        # the float tangent reductions group contributors by their position in the pattern, so a strand's
        # blocks sum in another association inside the batch: float rounding, not a different value
        ktol = 1e-12 if precision == "fp64" else 1e-6
        assert abs(Kbk - Kk).max() <= ktol * max(abs(Kk).max(), 1e-300), k
        # the instance's pairs in the batch table: elements shifted by e0
        hk = eng.pair_state()
        sel = (hb["ea"] >= e0) & (hb["ea"] < e1)
        assert np.array_equal(hb["ea"][sel] - e0, hk["ea"]) and np.array_equal(hb["eb"][sel] - e0, hk["eb"])
        assert np.array_equal(hb["status"][sel], hk["status"])
        assert np.array_equal(hb["stick"][sel], hk["stick"])
    assert pairs_total == sb["pairs"]
