"""K_c's block storage: the blocks with row <= column stand for the whole matrix (CPU).

Every contribution of a contact pair to K_c block (v, w) is c_k c_l B and the
same pair adds c_l c_k B to block (w, v), so the two blocks hold the same 3x3
values (not transposes: K_c is not symmetric once friction acts).  The
engine stores the blocks with row <= column only; ``to_csr`` rebuilds the
full matrix.  Checked on the oracle's K_c of the 7-wire strand with friction,
whose matrix is not symmetric.
"""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import contact as oc  # noqa: E402
from xkgpu import _lib as L  # noqa: E402
from xkgpu import workloads as W  # noqa: E402
from xkgpu.device import DeviceContactPattern  # noqa: E402


def _oracle_kc():
    w = W.config_workload("strand7", seed=0)
    st = w.strand
    n = st.ndof
    x = oc.deformed_coords(st.coords, w.u)
    t, _, _ = oc.detect(oc.empty_table(), x, st.conn, st.radii, elem_layer=st.elem_layer, exclude_same_layer=True)
    t = oc.update_geometry(t, x)
    rng = np.random.default_rng(3)
    u = w.u + rng.normal(0.0, 3e-4 * w.meta["d"], n) * np.tile([1, 1, 1, 0, 0, 0], st.n_nodes)
    _, _, Kc, _ = oc.contact_iteration(t, st.coords, u, w.u, n, k_pen=w.k_pen, k_t_ratio=w.k_t_ratio, mu_eff=w.mu)
    return Kc.toarray(), st.n_nodes


def test_mirrored_blocks_are_equal_and_rebuild_the_matrix():
    K, nn = _oracle_kc()
    scale = np.abs(K).max()
    assert np.abs(K - K.T).max() > 1e-6 * scale  # friction: not symmetric
    B = K.reshape(nn, 6, nn, 6)[:, :3, :, :3]  # B[v, :, w, :] = block (v, w)
    assert np.abs(B - B.transpose(2, 1, 0, 3)).max() <= 1e-14 * scale  # block (w, v) == block (v, w)
    nz = np.abs(B).max(axis=(1, 3)) > 0
    rows, cols = np.nonzero(np.triu(nz | nz.T))  # stored blocks: row <= column, (row, column) order
    pat = DeviceContactPattern.__new__(DeviceContactPattern)
    pat.c = L.ContactPattern()
    pat.c.nnzb = len(rows)
    pat.blk_row = torch.as_tensor(rows.astype(np.int32))
    pat.col = torch.as_tensor(cols.astype(np.int32))
    vals = torch.as_tensor(B[rows, :, cols, :].reshape(-1))
    full = pat.to_csr(vals, K.shape[0]).toarray()
    assert np.abs(full - K).max() <= 1e-14 * scale  # K_c has translational entries only


def test_beam_upper_blocks_rebuild_the_symmetric_tangent():
    """The reference symmetrises each element tangent (_beam_assembly.py:322): K_beam is stored as its
    row <= column 6x6 blocks, and ``DeviceBeam.to_csr`` puts the transposes below the diagonal."""
    from types import SimpleNamespace

    from oracle import beam as ob
    from xkgpu.device import DeviceBeam, make_beam_plan

    w = W.config_workload("strand7", seed=0)
    st = w.strand
    Kb, _ = ob.assemble_beam(st.coords, st.conn, w.u, ob.Section(**w.section, scf=None))
    K = Kb.toarray()
    assert np.array_equal(K, K.T)
    conn = np.array(st.conn)
    conn[::2] = conn[::2, ::-1]  # both element orientations: the lower block id is -1 on either side
    plan = make_beam_plan(conn, st.n_nodes)
    assert np.all((plan.blk[:, 1] < 0) == (conn[:, 0] > conn[:, 1]))
    assert np.all((plan.blk[:, 2] < 0) == (conn[:, 0] < conn[:, 1]))
    assert np.all(plan.first[:, None] >> np.arange(4) & 1 <= (plan.blk >= 0))
    rows = np.repeat(np.arange(st.n_nodes), np.diff(plan.row_ptr))
    assert np.all(rows <= plan.col)
    B = K.reshape(st.n_nodes, 6, st.n_nodes, 6)
    vals = torch.as_tensor(B[rows, :, plan.col, :].reshape(-1))
    beam = DeviceBeam.__new__(DeviceBeam)
    beam.plan_host = plan
    beam.mesh = SimpleNamespace(n_nodes=st.n_nodes, ndof=6 * st.n_nodes)
    assert np.array_equal(beam.to_csr(vals).toarray(), K)


def test_chain_order_detection():
    """The ordered one-launch float beam needs every wire's elements in sequence (element e's node b
    is element e+1's node a) or single-element wire ends; other chain meshes take the atomic form."""
    from xkgpu.device import chain_is_ordered

    wire = lambda n0, n: np.stack([n0 + np.arange(n), n0 + np.arange(1, n + 1)], 1)
    two = np.concatenate([wire(0, 5), wire(6, 3)])
    assert chain_is_ordered(two, 10)
    assert chain_is_ordered(np.array([[0, 1], [2, 3], [4, 5]]), 6)  # separate elements
    assert not chain_is_ordered(two[::-1], 10)                     # elements in reverse order
    assert not chain_is_ordered(two[[1, 0, 2, 3, 4, 5, 6, 7]], 10)  # two elements swapped
    assert not chain_is_ordered(np.array([[1, 0], [1, 2]]), 3)      # node 1 is node a of both
    assert not chain_is_ordered(np.zeros((0, 2), dtype=np.int64), 0)
    w = W.config_workload("strand7", seed=0)
    assert chain_is_ordered(w.strand.conn, w.strand.n_nodes)
