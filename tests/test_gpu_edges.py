"""Edge cases of the device assembly against the oracle (through the C ABI).

- No contact at all: two wires far apart, and a mesh of one element. The
  engine's residual and tangent are the beam's alone, eager and replayed.
- The pair table growing across detections, then every pair separating: the
  merge keeps the old pairs, adds the new ones in the reference's order, and
  the active-set hysteresis switches them off; the friction law still acts on
  separated pairs through their last normal pressure, as in the reference.
- A node touching more contact nodes than the pattern's row capacity: reported
  as an error status, not a fault.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err, sparse_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from oracle import beam as ob  # noqa: E402
from oracle import contact as oc  # noqa: E402
from xkgpu import _lib as L  # noqa: E402
from xkgpu import workloads as W  # noqa: E402
from xkgpu.engine import AssemblyEngine  # noqa: E402

TOL = {"fp64": 1e-10, "mixed": 1e-5}


def _dev(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def _section():
    return W.config_workload("strand7", seed=0).section


def _beam_only(coords, conn, u, sec):
    return ob.assemble_beam(coords, conn, u, ob.Section(**sec, scf=None))


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_no_contact_two_distant_wires(prec):
    z = np.linspace(0.0, 8.0, 9)
    coords = np.concatenate([np.stack([np.zeros(9), np.zeros(9), z], 1), np.stack([np.full(9, 10.0), np.zeros(9), z], 1)])
    conn = np.concatenate([np.stack([np.arange(8), np.arange(1, 9)], 1), 9 + np.stack([np.arange(8), np.arange(1, 9)], 1)])
    sec = _section()
    eng = AssemblyEngine(coords, conn, 0.3, sec, precision=prec, k_pen=1e4, mu=0.1)
    rng = np.random.default_rng(5)
    u = rng.normal(0.0, 1e-3, 6 * len(coords))
    stats = eng.detect(_dev(u))
    assert stats["pairs"] == 0 and stats["members"] == 0 and stats["contact_blocks"] == 0
    R = eng.assemble(_dev(u), _dev(u)).clone()
    torch.cuda.synchronize()
    Kb, fb = _beam_only(coords, conn, u, sec)
    assert rel_err(R.cpu().numpy(), fb) < TOL[prec]
    assert sparse_rel_err(eng.K_beam_csr(), Kb) < TOL[prec]
    assert eng.K_contact_csr().nnz == 0
    eng.capture(_dev(u), _dev(u))
    eng.replay()
    torch.cuda.synchronize()
    assert torch.equal(eng.R, R)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_single_element_mesh(prec):
    coords = np.array([[0.0, 0.0, 0.0], [0.3, 0.1, 1.0]])
    conn = np.array([[0, 1]])
    sec = _section()
    eng = AssemblyEngine(coords, conn, 0.5, sec, precision=prec, k_pen=1e4, mu=0.1)
    u = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.01, -0.02, 0.005, 0.3, -0.2, 0.1])
    assert eng.detect(_dev(u))["pairs"] == 0
    R = eng.assemble(_dev(u), _dev(u))
    torch.cuda.synchronize()
    Kb, fb = _beam_only(coords, conn, u, sec)
    assert rel_err(R.cpu().numpy(), fb) < TOL[prec]
    assert sparse_rel_err(eng.K_beam_csr(), Kb) < TOL[prec]


def _radial(st, factor):
    """Displacement that scales every node's distance from the strand axis by ``factor``."""
    c = st.coords[:, :2].mean(axis=0)
    u = np.zeros((st.n_nodes, 6))
    u[:, :2] = (factor - 1.0) * (st.coords[:, :2] - c)
    return u.ravel()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_table_growth_then_separation(prec):
    w = W.config_workload("strand7", seed=0)
    st = w.strand
    n = st.ndof
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=prec, **w.engine_kwargs())

    def oracle_detect(table, u):
        x = oc.deformed_coords(st.coords, u)
        t, _, _ = oc.detect(table, x, st.conn, st.radii, elem_layer=st.elem_layer, exclude_same_layer=True)
        return oc.update_geometry(t, x)

    def same_table(table):
        h = eng.pair_state()
        assert np.array_equal(h["ea"], table["ea"]) and np.array_equal(h["eb"], table["eb"])
        assert np.array_equal(h["status"], table["status"])

    # 1. wires pushed apart: few candidate pairs, none active
    u_far = _radial(st, 1.15)
    s1 = eng.detect(_dev(u_far))
    table = oracle_detect(oc.empty_table(), u_far)
    same_table(table)
    assert s1["members"] == 0
    # 2. the penetrating state: the table grows (new pairs appended in the reference's merge order)
    s2 = eng.detect(_dev(w.u))
    table = oracle_detect(table, w.u)
    same_table(table)
    assert s2["pairs"] > s1["pairs"] and s2["members"] > 0
    rng = np.random.default_rng(11)
    u = w.u + rng.normal(0.0, 2e-4 * w.meta["d"], n) * np.tile([1, 1, 1, 0, 0, 0], st.n_nodes)
    eng.assemble(_dev(u), _dev(w.u))
    torch.cuda.synchronize()
    table, fc, Kc, _ = oc.contact_iteration(table, st.coords, u, w.u, n, k_pen=w.k_pen, k_t_ratio=w.k_t_ratio,
                                            mu_eff=w.mu)
    Kb, fb = _beam_only(st.coords, st.conn, u, w.section)
    assert rel_err(eng.R.cpu().numpy(), fb + fc) < TOL[prec]
    assert sparse_rel_err(eng.K_contact_csr(), Kc) < TOL[prec]
    # stored blocks: row <= column; the lower index lists every off-diagonal one under its column
    pat = eng.pattern
    nb = pat.nnzb
    r, c = pat.blk_row[:nb].cpu().numpy(), pat.col[:nb].cpu().numpy()
    assert np.all(r <= c)
    lp = pat.low_ptr.cpu().numpy()
    lb = pat.low_blk[: lp[-1]].cpu().numpy()
    assert pat.nnzb_full == nb + int(np.sum(r != c)) == nb + lp[-1]
    assert np.array_equal(np.sort(lb), np.nonzero(r != c)[0])
    assert np.all(c[lb] == np.repeat(np.arange(st.n_nodes), np.diff(lp)))
    # 3. pushed apart again: every pair stays in the table and switches off
    eng.detect(_dev(u_far))
    table = oracle_detect(table, u_far)
    same_table(table)
    assert not np.any(table["status"] > 0)
    eng.assemble(_dev(u_far), _dev(u_far))
    torch.cuda.synchronize()
    _, fc, _, parts = oc.contact_iteration(table, st.coords, u_far, u_far, n, k_pen=w.k_pen,
                                           k_t_ratio=w.k_t_ratio, mu_eff=w.mu)
    _, fb = _beam_only(st.coords, st.conn, u_far, w.section)
    assert not np.any(parts["f_n"])  # no normal force once every pair is off
    # The normal law writes p_n of non-inactive pairs only, and the friction law runs over every pair
    # with p_n > 0 (strategy.py:126-170, _assembly.py:260-342): the separated pairs keep their last
    # p_n and so a friction force, which the device path reproduces.
    assert np.any(parts["f_f"])
    assert rel_err(eng.R.cpu().numpy(), fb + fc) < TOL[prec]


def test_pattern_row_capacity_is_an_error():
    """One element crossed by 300 short wires: each of its nodes touches 600 contact nodes (capacity 256)."""
    k = 300
    xs = -45.0 + 0.3 * np.arange(k)
    coords = [[-50.0, 0.0, 0.0], [50.0, 0.0, 0.0]]
    for x in xs:
        coords += [[x, -1.0, 0.9], [x, 1.0, 0.9]]
    coords = np.array(coords)
    conn = np.array([[0, 1]] + [[2 + 2 * i, 3 + 2 * i] for i in range(k)])
    eng = AssemblyEngine(coords, conn, 0.5, _section(), precision="fp64", k_pen=1e4, mu=0.0)
    with pytest.raises(L.XkError) as e:
        eng.detect(_dev(np.zeros(6 * len(coords))))
    assert e.value.code == L.XK_ERR_OVERFLOW and "256" in str(e.value)
    torch.cuda.synchronize()  # the context is still usable


def test_zero_length_element_is_refused():
    """An element whose two nodes coincide raises ValueError, as in the reference
    (elements/_beam_cr.py:50-56), before any beam kernel runs."""
    coords = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.0, 0.0, 1.0]])
    conn = np.array([[0, 1], [1, 2]])
    with pytest.raises(ValueError, match="zero length"):
        AssemblyEngine(coords, conn, 0.3, _section(), precision="mixed", k_pen=1e4, mu=0.1)
