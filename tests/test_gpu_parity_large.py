"""The GPU engine against the oracle at the benchmark configurations.

- the 91-wire strand (11,648 elements, ~108k pairs);
- the 1027-wire strand of the headline metric (98,592 elements, ~3.2M pairs);
- the 37-wire strand with its outer layer compressed radially by 0.005 d
  from the nominal lay (no minimum-gap bump);
- 16 strands of the 256-strand batch, each against its own oracle run.

Each case runs one detection from an empty pair table and two Newton
iterations on perturbed states, through the C ABI.  Candidate and active sets
are compared bit for bit (FP64 and mixed detection are both exact FP64);
residual R, beam tangent and contact tangent within 1e-10 (FP64) and 1e-5
(mixed) max-norm relative to the oracle's; stick flags and status equal.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err, sparse_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only hosts, skipped there
    pytest.skip("no CUDA device", allow_module_level=True)

from oracle import beam as ob  # noqa: E402
from oracle import contact as oc  # noqa: E402
from xkgpu import workloads as W  # noqa: E402
from xkgpu.engine import AssemblyEngine  # noqa: E402

TOL64, TOLMIX = 1e-10, 1e-5


def _dev(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def _states(st, u0, d, n_iter=2, seed=3):
    """The detection state and the Newton-iteration states (translations perturbed by 3e-4 d)."""
    rng = np.random.default_rng(seed)
    out, u = [], u0.copy()
    for _ in range(n_iter):
        u = u + rng.normal(0.0, 3e-4 * d, st.ndof) * np.tile([1, 1, 1, 0, 0, 0], st.n_nodes)
        out.append(u.copy())
    return out


def _oracle(st, section, u0, iters, *, k_pen, k_t_ratio, mu):
    """Detection + two iterations by the oracle: candidate set, active set, then per iteration
    (R, K_beam, K_c, status, stick)."""
    table, cands, raw = oc.detect(oc.empty_table(), oc.deformed_coords(st.coords, u0), st.conn, st.radii,
                                  elem_layer=st.elem_layer, exclude_same_layer=True)
    table = oc.update_geometry(table, oc.deformed_coords(st.coords, u0))
    ref = {"raw": len(raw), "cands": cands, "ea": table["ea"].copy(), "eb": table["eb"].copy(),
           "status0": table["status"].copy(), "iters": []}
    sec = ob.Section(**section, scf=None)
    for u in iters:
        table, fc, Kc, _ = oc.contact_iteration(table, st.coords, u, u0, st.ndof, k_pen=k_pen, k_t_ratio=k_t_ratio,
                                                mu_eff=mu)
        Kb, fb = ob.assemble_beam(st.coords, st.conn, u, sec)
        ref["iters"].append({"R": fb + fc, "Kb": Kb, "Kc": Kc, "status": table["status"].copy(),
                             "stick": table["stick"].copy()})
    return ref


def _check(eng, ref, u0, iters, tol):
    stats = eng.detect(_dev(u0))
    assert stats["raw"] == ref["raw"]
    assert stats["candidates"] == len(ref["cands"])
    h = eng.pair_state()
    assert np.array_equal(h["ea"], ref["ea"]) and np.array_equal(h["eb"], ref["eb"])
    assert np.array_equal(h["status"], ref["status0"])
    u_ref = _dev(u0)
    for u, r in zip(iters, ref["iters"]):
        eng.assemble(_dev(u), u_ref)
        torch.cuda.synchronize()
        h = eng.pair_state()
        assert np.array_equal(h["status"], r["status"])
        assert np.array_equal(h["stick"], r["stick"])
        assert rel_err(eng.R.cpu().numpy(), r["R"]) < tol
        assert sparse_rel_err(eng.K_contact_csr(), r["Kc"]) < tol
        assert sparse_rel_err(eng.K_beam_csr(), r["Kb"]) < tol


def _run_config(name, seed, precisions=("fp64", "mixed")):
    w = W.config_workload(name, seed=seed)
    st = w.strand
    iters = _states(st, w.u, w.meta["d"])
    ref = _oracle(st, w.section, w.u, iters, k_pen=w.k_pen, k_t_ratio=w.k_t_ratio, mu=w.mu)
    assert len(ref["cands"]) > 0 and int((ref["status0"] != 0).sum()) > 0
    for precision in precisions:
        eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=precision, **w.engine_kwargs())
        _check(eng, ref, w.u, iters, TOL64 if precision == "fp64" else TOLMIX)
        del eng
        torch.cuda.empty_cache()
    return ref


def test_strand91_vs_oracle():
    """C3's 91-wire strand (4 pitches x 32 elements per wire)."""
    ref = _run_config("strand91", seed=1)
    assert len(ref["cands"]) > 100_000


def test_strand37_compressed_vs_oracle():
    """C2's 37-wire strand, outer layer pushed radially inward by 0.005 d from the nominal lay."""
    w = W.config_workload("strand37c", seed=2)
    assert w.meta["compress_layer"] == 3 and w.meta["compress_frac"] == 0.005
    ref = _run_config("strand37c", seed=2)
    # the compression is what makes contact: layer 3 is in every active pair with layer 2
    st = w.strand
    act = ref["status0"] != 0
    la, lb = st.elem_layer[ref["ea"][act]], st.elem_layer[ref["eb"][act]]
    assert np.any((np.minimum(la, lb) == 2) & (np.maximum(la, lb) == 3))


def test_strand1027_vs_oracle():
    """The headline configuration, whole: 1027 wires, ~100k nodes, ~3.2M pairs, ~750k contributing."""
    ref = _run_config("strand1027", seed=1)
    assert len(ref["cands"]) > 3_000_000
    assert int((ref["status0"] != 0).sum()) > 700_000


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch256_sample_vs_oracle(precision):
    """The 256-strand batch assembled as one mesh; 16 of its strands, each against a separate oracle run
    on that strand alone with its own friction coefficient."""
    w = W.config_workload("batch256", seed=0)
    st = w.strand
    inst, first = w.meta["instance"], w.meta["node_first"]
    mus = w.meta["mu_instance"]
    d = w.meta["d"]
    iters = _states(st, w.u, d, n_iter=1)
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, layer=st.elem_layer, precision=precision,
                         k_pen=w.k_pen, mu=w.mu)
    eng.detect(_dev(w.u))
    eng.assemble(_dev(iters[0]), _dev(w.u))
    torch.cuda.synchronize()
    R = eng.R.cpu().numpy()
    Kc = eng.K_contact_csr()
    Kb = eng.K_beam_csr()
    h = eng.pair_state()
    tol = TOL64 if precision == "fp64" else TOLMIX
    bounds = list(first) + [st.n_nodes]
    sample = np.random.default_rng(5).choice(len(first), 16, replace=False)
    sec = ob.Section(**w.section, scf=None)
    for k in sorted(int(x) for x in sample):
        n0, n1 = int(bounds[k]), int(bounds[k + 1])
        el = np.nonzero(inst == k)[0]
        e0, e1 = int(el[0]), int(el[-1]) + 1
        X, conn = st.coords[n0:n1], st.conn[e0:e1] - n0
        u0, u1 = w.u[6 * n0:6 * n1], iters[0][6 * n0:6 * n1]
        ndof = 6 * (n1 - n0)
        table, cands, _ = oc.detect(oc.empty_table(), oc.deformed_coords(X, u0), conn, st.radii[e0:e1],
                                    elem_layer=st.elem_layer[e0:e1], exclude_same_layer=True)
        table = oc.update_geometry(table, oc.deformed_coords(X, u0))
        table, fc, Kck, _ = oc.contact_iteration(table, X, u1, u0, ndof, k_pen=w.k_pen, k_t_ratio=w.k_t_ratio,
                                                 mu_eff=float(mus[k]))
        Kbk, fb = ob.assemble_beam(X, conn, u1, sec)
        sel = (h["ea"] >= e0) & (h["ea"] < e1)
        assert np.array_equal(h["ea"][sel] - e0, table["ea"]) and np.array_equal(h["eb"][sel] - e0, table["eb"])
        assert np.array_equal(h["status"][sel], table["status"]), k
        assert np.array_equal(h["stick"][sel], table["stick"]), k
        assert rel_err(R[6 * n0:6 * n1], fb + fc) < tol, k
        assert sparse_rel_err(Kc[6 * n0:6 * n1, 6 * n0:6 * n1], Kck) < tol, k
        assert sparse_rel_err(Kb[6 * n0:6 * n1, 6 * n0:6 * n1], Kbk) < tol, k


@pytest.mark.parametrize("end_rotation", [None, 0.5])
def test_mixed_at_large_rotation_bent_strand(end_rotation):
    """The mixed engine against the FP64 engine and the oracle on the 91-wire strand bent into an arc:
    curvature 1/(50 D) (end sections turned by 0.15 rad), or an arc whose ends turn by 0.5 rad; every
    element rotates rigidly by up to that angle with little deformation, plus the seeded noise.
    R, K_beam and K_c within 1e-5 (max-norm relative), active and stick sets equal."""
    from xkgpu import runs

    w = W.config_workload("strand91", seed=4)
    st = w.strand
    D = 2.0 * max(wi.lay_radius for wi in st.wires) + w.meta["d"]
    kappa = 1.0 / (50.0 * D) if end_rotation is None else end_rotation / st.length
    u0 = w.u + runs.arc_displacement(st, kappa)
    assert np.max(np.abs(u0.reshape(-1, 6)[:, 3])) > 0.9 * kappa * st.length
    iters = _states(st, u0, w.meta["d"], n_iter=1)
    ref = _oracle(st, w.section, u0, iters, k_pen=w.k_pen, k_t_ratio=w.k_t_ratio, mu=w.mu)
    out = {}
    for precision in ("fp64", "mixed"):
        eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=precision, **w.engine_kwargs())
        _check(eng, ref, u0, iters, TOL64 if precision == "fp64" else TOLMIX)
        out[precision] = (eng.R.cpu().numpy(), eng.K_beam_csr(), eng.K_contact_csr())
    for a, b in zip(out["mixed"], out["fp64"]):
        err = rel_err(a, b) if isinstance(a, np.ndarray) else sparse_rel_err(a, b)
        assert err < TOLMIX


@pytest.mark.parametrize("name", ["strand91", "strand1027"])
def test_screened_detection_equals_exact(name):
    """The mixed engine's detection decides the active set in float wherever the float gap is provably on
    the same side of the thresholds (``xk_narrowphase_screened``): the status of every pair equals the
    exact routine's, the float gaps of the other pairs are within 2e-5 of the segment scale of the exact
    ones, and only a small share of the pairs needs the exact routine."""
    w = W.config_workload(name, seed=6)
    st = w.strand
    u = _dev(w.u)
    out = {}
    for screened in (False, True):
        eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="mixed", **w.engine_kwargs())
        eng.screened_detection = screened
        stats = eng.detect(u)
        out[screened] = (eng.pair_state(), stats)
        del eng
    ex, sc = out[False][0], out[True][0]
    assert np.array_equal(ex["ea"], sc["ea"]) and np.array_equal(ex["eb"], sc["eb"])
    assert np.array_equal(ex["status"], sc["status"])
    n_exact = out[True][1]["narrowphase_exact"]
    assert n_exact < 0.05 * len(ex["ea"])
    assert np.max(np.abs(ex["gap"] - sc["gap"])) < 2e-5 * 2.0 * w.meta["d"]
    near = np.abs(ex["gap"]) < 1e-4
    print(f"{name}: {len(ex['ea'])} pairs, {n_exact} exact, {int(near.sum())} within 1e-4 of contact, "
          f"max |gap float - gap exact| = {np.max(np.abs(ex['gap'] - sc['gap'])):.3e}")
