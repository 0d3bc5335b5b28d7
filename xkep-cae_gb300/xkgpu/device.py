"""Device-resident data of the assembly path: mesh, beam plan, pair table, contact pattern.

PyTorch supplies device memory and the CUDA stream; all arithmetic runs in the
xkgpu kernels behind the C ABI.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib as L

INACTIVE, ACTIVE, SLIDING = 0, 1, 2


def require_cuda(device=None) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("xkgpu needs a CUDA device: no GPU is visible to this process")
    L.load()
    return torch.device(device if device is not None else "cuda")


def stream_handle(stream=None) -> C.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def ptr(t: torch.Tensor | None) -> C.c_void_p:
    return C.c_void_p(0 if t is None else t.data_ptr())


def as_dev(x, dtype, device) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.array(x, copy=True, order="C"), dtype=dtype, device=device)


# ----------------------------------------------------------------------------- mesh


class DeviceMesh:
    """Reference coordinates, connectivity, radii and layer ids on the device."""

    def __init__(self, coords, conn, radii, layer=None, device=None, mu=None, core_radii=None):
        self.device = require_cuda(device)
        coords = np.asarray(coords, dtype=np.float64).reshape(-1, 3)
        conn = np.asarray(conn, dtype=np.int64).reshape(-1, 2)
        self.n_nodes = int(coords.shape[0])
        self.n_elems = int(conn.shape[0])
        radii = np.broadcast_to(np.asarray(radii, dtype=np.float64), (self.n_elems,))
        if self.n_elems and (conn.min() < 0 or conn.max() >= self.n_nodes):
            raise ValueError("connectivity refers to nodes outside [0, n_nodes)")
        if layer is not None and np.asarray(layer).shape[0] != self.n_elems:
            raise ValueError("layer must hold one entry per element")
        self.X = as_dev(coords.ravel(), torch.float64, self.device)
        self.conn = as_dev(conn.ravel().astype(np.int32), torch.int32, self.device)
        self.radii = as_dev(radii, torch.float64, self.device)
        self.layer = None if layer is None else as_dev(np.asarray(layer).astype(np.int32), torch.int32, self.device)
        if mu is not None and np.asarray(mu).shape != (self.n_elems,):
            raise ValueError("mu must hold one friction coefficient per element")
        self.mu = None if mu is None else as_dev(np.asarray(mu, dtype=np.float64), torch.float64, self.device)
        # coated wires: the core radius of every element (the narrowphase's gap is between the cores)
        self.core_radii = None if core_radii is None else as_dev(
            np.broadcast_to(np.asarray(core_radii, dtype=np.float64), (self.n_elems,)).copy(), torch.float64,
            self.device)
        self.conn_host = conn
        self.refresh()

    def refresh(self):
        self.c = L.Mesh(self.n_nodes, self.n_elems, ptr(self.X), ptr(self.conn), ptr(self.radii), ptr(self.layer),
                        ptr(self.mu), ptr(self.core_radii))

    def set_coords(self, coords):
        self.X.copy_(as_dev(np.asarray(coords, dtype=np.float64).ravel(), torch.float64, self.device))

    @property
    def ndof(self) -> int:
        return 6 * self.n_nodes


# ----------------------------------------------------------------------------- beam plan


def beam_block_pattern(conn: np.ndarray, n_nodes: int):
    """6x6 block-CSR pattern of the beam tangent's stored blocks and each element's 4 block ids.

    The structural pattern of ``assemble_cr_beam3d``'s CSR
    (``_beam_assembly.py:146-150``) in 6x6 blocks is (a,a), (a,b), (b,a), (b,b)
    of every element a-b.  The reference symmetrises every element tangent
    (``_beam_assembly.py:322``), so block (w, v) is the transpose of block
    (v, w): only the blocks with row <= column are stored, rows sorted by
    column, and the element's id of its other off-diagonal block is -1.
    """
    conn = np.asarray(conn, dtype=np.int64)
    a, b = conn[:, 0], conn[:, 1]
    rows = np.stack([a, a, b, b], axis=1)
    cols = np.stack([a, b, a, b], axis=1)
    keys = rows * n_nodes + cols
    upper = rows <= cols
    uk = np.unique(keys[upper])
    brow = uk // n_nodes
    bcol = (uk % n_nodes).astype(np.int32)
    row_ptr = np.zeros(n_nodes + 1, dtype=np.int64)
    np.add.at(row_ptr, brow + 1, 1)
    row_ptr = np.cumsum(row_ptr)
    blk = np.where(upper, np.searchsorted(uk, keys), -1).astype(np.int32)
    return row_ptr.astype(np.int32), bcol, blk


def lower_index(row_ptr: np.ndarray, col: np.ndarray, n_nodes: int):
    """Per node w, the stored blocks (v, w) with v < w, ascending in v: (blk_row, low_ptr, low_blk)."""
    rows = np.repeat(np.arange(n_nodes, dtype=np.int64), np.diff(row_ptr))
    off = np.nonzero(rows != col)[0]
    order = np.lexsort((rows[off], col[off]))
    low_blk = off[order].astype(np.int32)
    low_ptr = np.zeros(n_nodes + 1, dtype=np.int64)
    np.add.at(low_ptr, col[off].astype(np.int64) + 1, 1)
    return rows.astype(np.int32), np.cumsum(low_ptr).astype(np.int32), low_blk


def greedy_coloring(conn: np.ndarray, n_nodes: int) -> np.ndarray:
    """Colour elements so that no two elements of one colour share a node."""
    conn = np.asarray(conn, dtype=np.int64)
    ne = conn.shape[0]
    colors = np.empty(ne, dtype=np.int32)
    used: list[set] = [set() for _ in range(n_nodes)]
    for e in range(ne):
        a, b = int(conn[e, 0]), int(conn[e, 1])
        forbid = used[a] | used[b]
        c = 0
        while c in forbid:
            c += 1
        colors[e] = c
        used[a].add(c)
        used[b].add(c)
    return colors


@dataclass
class BeamPlanHost:
    row_ptr: np.ndarray
    col: np.ndarray
    blk: np.ndarray  # (n_elems, 4)
    colors: np.ndarray
    order: np.ndarray
    color_ptr: np.ndarray
    first: np.ndarray  # (n_elems,) uint8 bits

    @property
    def nnzb(self) -> int:
        return int(self.col.shape[0])


def make_beam_plan(conn: np.ndarray, n_nodes: int) -> BeamPlanHost:
    row_ptr, col, blk = beam_block_pattern(conn, n_nodes)
    colors = greedy_coloring(conn, n_nodes)
    order = np.argsort(colors, kind="stable").astype(np.int32)
    ncol = int(colors.max()) + 1 if colors.size else 0
    color_ptr = np.zeros(ncol + 1, dtype=np.int32)
    np.add.at(color_ptr, colors + 1, 1)
    color_ptr = np.cumsum(color_ptr).astype(np.int32)
    # first writer of each block: the element of the lowest colour touching it
    nblk = col.shape[0]
    best = np.full(nblk, np.iinfo(np.int32).max, dtype=np.int64)
    ecol = np.repeat(colors[:, None], 4, axis=1)
    stored = blk >= 0
    np.minimum.at(best, blk[stored], ecol[stored])
    isfirst = stored & (ecol == best[np.where(stored, blk, 0)])
    first = (isfirst * (1 << np.arange(4))[None, :]).sum(axis=1).astype(np.uint8)
    return BeamPlanHost(row_ptr, col, blk, colors, order, color_ptr, first)


def chain_node_diag(conn: np.ndarray, n_nodes: int, plan: BeamPlanHost) -> np.ndarray | None:
    """Diagonal block of every node (-1 without element) if the mesh is a set of chains, else None.

    A chain mesh has at most two elements at every node and no two elements on
    the same pair of nodes, so that every shared location of K_T and f_int has
    exactly two contributions."""
    conn = np.asarray(conn, dtype=np.int64)
    if conn.shape[0] == 0 or np.any(conn[:, 0] == conn[:, 1]):
        return None
    if np.bincount(conn.ravel(), minlength=n_nodes).max() > 2:
        return None
    key = np.sort(conn, axis=1)
    if np.unique(key[:, 0] * n_nodes + key[:, 1]).shape[0] != conn.shape[0]:
        return None
    diag = np.full(n_nodes, -1, dtype=np.int32)
    diag[conn[:, 0]] = plan.blk[:, 0]
    diag[conn[:, 1]] = plan.blk[:, 3]
    return diag


def chain_is_ordered(conn: np.ndarray, n_nodes: int) -> bool:
    """Whether the elements of a chain mesh follow each other along every wire: node b of element e
    is node a of element e + 1, or the node belongs to one element only (a wire end)."""
    conn = np.asarray(conn, dtype=np.int64)
    if conn.shape[0] == 0:
        return False
    a, b = conn[:, 0], conn[:, 1]
    cnt = np.bincount(conn.ravel(), minlength=n_nodes)
    joined = np.zeros(a.shape[0], dtype=bool)
    joined[1:] = b[:-1] == a[1:]  # element e continues element e - 1
    ok_a = (cnt[a] == 1) | (joined & (cnt[a] == 2))
    nxt = np.zeros(a.shape[0], dtype=bool)
    nxt[:-1] = joined[1:]
    ok_b = (cnt[b] == 1) | (nxt & (cnt[b] == 2))
    return bool(np.all(ok_a & ok_b))


class DeviceBeam:
    """CR beam data: section, per-element reference frames and the K_T plan."""

    def __init__(self, mesh: DeviceMesh, section: dict, *, v_ref=None, chain: bool = True):
        self.mesh = mesh
        dev = mesh.device
        scf = section.get("scf")
        self.section = L.Section(section["E"], section["G"], section["A"], section["Iy"], section["Iz"],
                                 section["J"], section["kappa_y"], section["kappa_z"],
                                 float(scf) if scf is not None and scf > 0 else 0.0)
        self.v_ref = None if v_ref is None else np.asarray(v_ref, dtype=np.float64)
        self.plan_host = make_beam_plan(mesh.conn_host, mesh.n_nodes)
        ph = self.plan_host
        self.order = torch.as_tensor(ph.order, device=dev)
        self.blk = torch.as_tensor(ph.blk.ravel(), device=dev)
        self.first = torch.as_tensor(ph.first, device=dev)
        self.row_ptr = torch.as_tensor(ph.row_ptr, device=dev)
        self.col = torch.as_tensor(ph.col, device=dev)
        brow, lptr, lblk = lower_index(ph.row_ptr, ph.col, mesh.n_nodes)
        self.blk_row = torch.as_tensor(brow, device=dev)
        self.low_ptr = torch.as_tensor(lptr, device=dev)
        self.low_blk = torch.as_tensor(lblk if lblk.size else np.zeros(1, np.int32), device=dev)
        self._color_ptr = (C.c_int32 * len(ph.color_ptr))(*ph.color_ptr.tolist())
        # wires: every node in at most two elements, no two elements on the same nodes -> one-launch float path
        nd = chain_node_diag(mesh.conn_host, mesh.n_nodes, ph) if chain else None
        self.node_diag = None if nd is None else torch.as_tensor(nd, device=dev)
        self.chain_ordered = nd is not None and chain_is_ordered(mesh.conn_host, mesh.n_nodes)
        # beam_ctas_per_sm (last field) 0: the float beam's full grid.  A cap of 1-3 CTAs per SM, which lets
        # it share the SMs with the pair kernels, measured 1% faster per step at the 1027-wire strand
        # (0.1819-0.1830 against 0.1839 ms); the full grid stays the default, so that the beam launch on its
        # own keeps its one-wave time.
        self.plan = L.BeamPlan(len(ph.color_ptr) - 1, C.cast(self._color_ptr, C.c_void_p), ptr(self.order),
                               ptr(self.blk), ptr(self.first), ph.nnzb, ptr(self.node_diag),
                               int(self.chain_ordered), 0)
        self.elem_ref = torch.empty(10 * max(mesh.n_elems, 1), dtype=torch.float64, device=dev)
        self.update_reference_frames()

    def check_lengths(self):
        """Raise ValueError for an element whose two nodes coincide (length < 1e-15), as the reference
        does (``_beam3d_length_and_direction``, ``elements/_beam_cr.py:50-56``)."""
        if self.mesh.n_elems == 0:
            return
        X = self.mesh.X.view(-1, 3)
        c = self.mesh.conn.view(-1, 2).long()
        L = torch.linalg.vector_norm(X[c[:, 1]] - X[c[:, 0]], dim=1)
        bad = torch.nonzero(L < 1e-15)
        if bad.numel():
            raise ValueError(f"element {int(bad[0, 0])} has (almost) zero length: its two nodes coincide")

    def update_reference_frames(self, stream=None):
        self.check_lengths()
        vr = None if self.v_ref is None else (C.c_double * 3)(*self.v_ref.tolist())
        L.call("xk_beam_reference", C.byref(self.mesh.c), vr, ptr(self.elem_ref), stream_handle(stream))

    def assemble(self, u: torch.Tensor, precision: int, f_int: torch.Tensor | None, K_vals: torch.Tensor | None,
                 stream=None):
        L.call("xk_beam_assemble", C.byref(self.mesh.c), C.byref(self.section), ptr(self.elem_ref),
               C.byref(self.plan), ptr(u), precision, ptr(f_int), ptr(K_vals), stream_handle(stream))

    def lumped_mass(self, rho: float, out: torch.Tensor, stream=None):
        L.call("xk_beam_lumped_mass", C.byref(self.mesh.c), C.byref(self.section), C.byref(self.plan),
               float(rho), ptr(out), stream_handle(stream))

    @property
    def nnzb(self) -> int:
        return self.plan_host.nnzb

    def to_csr(self, vals: torch.Tensor) -> sp.csr_matrix:
        """The full beam tangent (ndof x ndof CSR) from its stored (row <= column) 6x6 blocks: every
        off-diagonal stored block (v, w) stands transposed at (w, v)."""
        ph = self.plan_host
        nb = ph.nnzb
        nd = self.mesh.ndof
        v = vals[: 36 * nb].double().cpu().numpy().reshape(nb, 6, 6)
        r = np.repeat(np.arange(self.mesh.n_nodes, dtype=np.int64), np.diff(ph.row_ptr))
        c = ph.col.astype(np.int64)
        off = r != c
        r, c = np.concatenate([r, c[off]]), np.concatenate([c, r[off]])
        v = np.concatenate([v, v[off].transpose(0, 2, 1)])
        rows = np.broadcast_to((6 * r)[:, None, None] + np.arange(6)[None, :, None], v.shape)
        cols = np.broadcast_to((6 * c)[:, None, None] + np.arange(6)[None, None, :], v.shape)
        return sp.csr_matrix((v.ravel(), (rows.ravel(), cols.ravel())), shape=(nd, nd))

    def diag_index(self) -> torch.Tensor:
        """Value index (into the 6x6 block values) of every DOF's diagonal entry; -1 for a node without elements."""
        if getattr(self, "_diag_index", None) is None:
            ph = self.plan_host
            n = self.mesh.n_nodes
            rows = np.repeat(np.arange(n), np.diff(ph.row_ptr))
            db = np.nonzero(ph.col == rows)[0]
            idx = np.full((n, 6), -1, dtype=np.int64)
            idx[rows[db]] = 36 * db[:, None] + 7 * np.arange(6)[None, :]
            self._diag_index = torch.as_tensor(idx.ravel(), device=self.mesh.device)
        return self._diag_index

    def k_dtype(self, precision: int):
        return torch.float64 if precision == L.XK_FP64 else torch.float32


# ----------------------------------------------------------------------------- pair table

F64_FIELDS = {"s": 1, "t": 1, "gap": 1, "normal": 3, "t1": 3, "t2": 3, "lambda_n": 1, "k_pen": 1, "k_t": 1,
              "p_n": 1, "z_t": 2, "q_trial_norm": 1, "dissipation": 1}
U8_FIELDS = ("status", "stick")
# coating state of coated wires (double, then the stick flag)
COAT_F64 = {"coat_cc": 1, "coat_cc_prev": 1, "coat_z_t": 2, "coat_qtn": 1, "coat_diss": 1}
COAT_U8 = ("coat_stick",)


class DevicePairTable:
    """Structure-of-arrays pair table (``xk_pairs``), vector fields component-major."""

    def __init__(self, device, cap: int = 1024, coating: bool = False):
        self.device = device
        self.n = 0
        self.cap = 0
        self.coating = coating  # the table carries the coating state (coated wires)
        self.t: dict[str, torch.Tensor] = {}
        self.reserve(max(cap, 16))

    def _f64(self):
        return {**F64_FIELDS, **COAT_F64} if self.coating else F64_FIELDS

    def _u8(self):
        return (*U8_FIELDS, *COAT_U8) if self.coating else U8_FIELDS

    def reserve(self, cap: int, keep: bool = True):
        if cap <= self.cap:
            return
        cap = int(cap)
        new = {"ea": torch.zeros(cap, dtype=torch.int32, device=self.device),
               "eb": torch.zeros(cap, dtype=torch.int32, device=self.device)}
        for k, w in self._f64().items():
            new[k] = torch.zeros(w * cap, dtype=torch.float64, device=self.device)
        for k in self._u8():
            new[k] = torch.zeros(cap, dtype=torch.uint8, device=self.device)
        if keep and self.n:
            n, oc = self.n, self.cap
            for k in ("ea", "eb", *self._u8()):
                new[k][:n] = self.t[k][:n]
            for k, w in self._f64().items():
                for c in range(w):
                    new[k][c * cap : c * cap + n] = self.t[k][c * oc : c * oc + n]
        self.t = new
        self.cap = cap
        self.refresh()

    def refresh(self):
        t = self.t
        self.c = L.Pairs(self.n, self.cap, *(ptr(t[k]) for k in (
            "ea", "eb", "s", "t", "gap", "normal", "t1", "t2", "lambda_n", "k_pen", "k_t", "p_n", "z_t",
            "q_trial_norm", "dissipation", "status", "stick")), *(ptr(t.get(k)) for k in L.COAT64_FIELDS))

    def set_n(self, n: int):
        self.n = int(n)
        self.c.n = self.n

    def to_host(self) -> dict:
        """Copy the table to host arrays in the oracle's layout (for checks and strategies)."""
        n, cap = self.n, self.cap
        out = {"ea": self.t["ea"][:n].cpu().numpy().astype(np.int64),
               "eb": self.t["eb"][:n].cpu().numpy().astype(np.int64)}
        for k, w in self._f64().items():
            a = self.t[k].view(w, cap)[:, :n].cpu().numpy() if w > 1 else self.t[k][:n].cpu().numpy()
            out[k] = a.T.copy() if w > 1 else a.copy()
        out["status"] = self.t["status"][:n].cpu().numpy().astype(np.int8)
        out["stick"] = self.t["stick"][:n].cpu().numpy().astype(bool)
        if self.coating:
            out["coat_stick"] = self.t["coat_stick"][:n].cpu().numpy().astype(bool)
        return out

    def from_host(self, d: dict, n_elems: int | None = None):
        n = int(np.asarray(d["ea"]).shape[0])
        if n_elems is not None and n and (min(np.min(d["ea"]), np.min(d["eb"])) < 0
                                          or max(np.max(d["ea"]), np.max(d["eb"])) >= n_elems):
            raise ValueError("pair table refers to elements outside [0, n_elems)")
        self.reserve(n, keep=False)
        cap = self.cap
        self.t["ea"][:n] = torch.as_tensor(np.asarray(d["ea"], dtype=np.int32), device=self.device)
        self.t["eb"][:n] = torch.as_tensor(np.asarray(d["eb"], dtype=np.int32), device=self.device)
        for k, w in self._f64().items():
            if k not in d:  # coating state absent from the source: fresh (zero)
                continue
            a = np.asarray(d[k], dtype=np.float64).reshape(n, w) if w > 1 else np.asarray(d[k], dtype=np.float64)
            if w > 1:
                self.t[k].view(w, cap)[:, :n] = torch.as_tensor(a.T.copy(), device=self.device)
            else:
                self.t[k][:n] = torch.as_tensor(a, device=self.device)
        self.t["status"][:n] = torch.as_tensor(np.asarray(d["status"]).astype(np.uint8), device=self.device)
        self.t["stick"][:n] = torch.as_tensor(np.asarray(d["stick"]).astype(np.uint8), device=self.device)
        if self.coating:
            self.t["coat_stick"][:n] = torch.as_tensor(np.asarray(d.get("coat_stick", np.ones(n, bool)))
                                                       .astype(np.uint8), device=self.device)
        self.set_n(n)
        self.refresh()

    def copy_from(self, other: "DevicePairTable"):
        self.reserve(other.n, keep=False)
        n, cap, oc = other.n, self.cap, other.cap
        for k in ("ea", "eb", *self._u8()):
            self.t[k][:n] = other.t[k][:n]
        for k, w in self._f64().items():
            for c in range(w):
                self.t[k][c * cap : c * cap + n] = other.t[k][c * oc : c * oc + n]
        self.set_n(n)
        self.refresh()


F32_FIELDS = {"rad": 2, "s": 1, "t": 1, "gap": 1, "normal": 3, "t1": 3, "t2": 3, "p_n": 1, "z_t": 2,
              "q_trial_norm": 1, "dissipation": 1, "k_pen": 1, "k_t": 1}


class DevicePairTable32:
    """Slot-ordered float copy of the pair state (``xk_pairs32``) for the mixed per-iteration kernels."""

    def __init__(self, device, per_slot_mu: bool = False, coating: bool = False):
        self.device = device
        self.cap = 0
        self.t: dict[str, torch.Tensor] = {}
        self.c = L.Pairs32()
        self.per_slot_mu = per_slot_mu  # the mesh has a friction coefficient per element
        self.coating = coating  # coated wires: coat_total and the coating state per slot

    def ensure(self, cap: int):
        if cap <= self.cap:
            return
        cap = int(cap)
        t = {"pair": torch.zeros(cap, dtype=torch.int32, device=self.device),
             "nodes": torch.zeros(4 * cap, dtype=torch.int32, device=self.device)}
        t.update({k: torch.zeros(w * cap, dtype=torch.float32, device=self.device) for k, w in F32_FIELDS.items()})
        t["status"] = torch.zeros(cap, dtype=torch.uint8, device=self.device)
        t["stick"] = torch.zeros(cap, dtype=torch.uint8, device=self.device)
        t["mu"] = torch.zeros(cap, dtype=torch.float32, device=self.device) if self.per_slot_mu else None
        t["defer"] = torch.zeros(2 * (cap + 2), dtype=torch.int32, device=self.device)
        t["slot"] = torch.zeros(cap, dtype=torch.int32, device=self.device)
        if self.coating:
            for k, w in (("coat_total", 1), ("coat_cc", 1), ("coat_cc_prev", 1), ("coat_z_t", 2), ("coat_qtn", 1),
                         ("coat_diss", 1)):
                t[k] = torch.zeros(w * cap, dtype=torch.float32, device=self.device)
            t["coat_stick"] = torch.zeros(cap, dtype=torch.uint8, device=self.device)
        self.t = t
        self.cap = cap
        self.c = L.Pairs32(0, cap, 0, *(ptr(t[k]) for k in (
            "pair", "nodes", "rad", "s", "t", "gap", "normal", "t1", "t2", "p_n", "z_t", "q_trial_norm",
            "dissipation", "k_pen", "k_t", "status", "stick", "mu")), *(ptr(t.get(k)) for k in L.COAT32_FIELDS),
            ptr(t["defer"]))
        self.c.slot = ptr(t["slot"])


# ----------------------------------------------------------------------------- contact pattern


class DeviceContactPattern:
    """Members / other pairs, member incidence, K_c block pattern and contributor lists."""

    GROW = 1.25

    def __init__(self, mesh: DeviceMesh):
        self.mesh = mesh
        self.c = L.ContactPattern()
        self.inc_ptr = self._i32(mesh.n_nodes + 1)
        self.row_ptr = self._i32(mesh.n_nodes + 1)
        self.low_ptr = self._i32(mesh.n_nodes + 1)
        # element-side form (mesh topology, element incidence, cross lists, element sums)
        self.node_elem_ptr = self._i32(mesh.n_nodes + 1)
        self.node_elem = self._i32(4 * mesh.n_elems)
        self.elem_ptr = self._i32(mesh.n_elems + 1)
        self.elem_sums = torch.zeros(56 * max(mesh.n_elems, 1), dtype=torch.float64, device=mesh.device)
        self.norm_scratch = torch.zeros((6 * mesh.n_nodes + 255) // 256 + 1, dtype=torch.float64,
                                        device=mesh.device)
        self._alloc_members(256)
        self._alloc_others(256)
        self._alloc_blocks(1024)
        self.version = 0

    def _i32(self, n):
        return torch.zeros(max(int(n), 1), dtype=torch.int32, device=self.mesh.device)

    def _alloc_members(self, cap):
        cap = int(cap)
        self.members, self.member_nodes = self._i32(cap), self._i32(4 * cap)
        self.inc, self.contrib = self._i32(4 * cap), self._i32(16 * cap)
        self.elem_inc = self._i32(2 * cap)
        self.cap_members = cap

    def _alloc_others(self, cap):
        self.others = self._i32(cap)
        self.cap_others = int(cap)

    def _alloc_blocks(self, cap):
        cap = int(cap)
        self.col, self.blk_row, self.blk_ptr = self._i32(cap), self._i32(cap), self._i32(cap + 1)
        self.low_blk = self._i32(cap)
        self.bcodes = self._i32(4 * cap)
        self.cap_blocks = cap

    def _sync_struct(self):
        c = self.c
        c.n_nodes = self.mesh.n_nodes
        c.cap_members, c.cap_others, c.cap_blocks = self.cap_members, self.cap_others, self.cap_blocks
        for k in ("members", "member_nodes", "others", "inc_ptr", "inc", "row_ptr", "col", "blk_row", "blk_ptr",
                  "contrib", "node_elem_ptr", "node_elem", "elem_ptr", "elem_inc", "bcodes", "elem_sums",
                  "norm_scratch", "low_ptr", "low_blk"):
            setattr(c, k, ptr(getattr(self, k)))

    def build(self, pairs: DevicePairTable, stream=None):
        for _ in range(4):
            self._sync_struct()
            code = L.call("xk_contact_pattern_build", C.byref(self.mesh.c), C.byref(pairs.c), C.byref(self.c),
                          stream_handle(stream), allow=(L.XK_ERR_CAPACITY,))
            if code == L.XK_OK:
                self.version += 1
                return
            if self.c.n_members > self.cap_members:
                self._alloc_members(self.c.n_members * self.GROW + 64)
            if self.c.n_others > self.cap_others:
                self._alloc_others(self.c.n_others * self.GROW + 64)
            if self.c.nnzb > self.cap_blocks:
                self._alloc_blocks(self.c.nnzb * self.GROW + 64)
        raise RuntimeError("contact pattern capacity did not converge")

    @property
    def n_members(self) -> int:
        return int(self.c.n_members)

    @property
    def nnzb(self) -> int:
        return int(self.c.nnzb)

    @property
    def n_contrib(self) -> int:
        return int(self.c.n_contrib)

    @property
    def nnzb_full(self) -> int:
        """Blocks of the full K_c: the stored (row <= column) blocks and the mirrors of the off-diagonal ones."""
        return int(self.c.nnzb_full)

    def to_csr(self, vals: torch.Tensor, ndof: int, drop_tiny: bool = False) -> sp.csr_matrix:
        """The full K_c (ndof x ndof CSR) from the stored blocks' values (9 per block): every off-diagonal
        stored block (v, w) also stands at (w, v), with the same values."""
        nb = self.nnzb
        if nb == 0:
            return sp.csr_matrix((ndof, ndof))
        v = vals[: 9 * nb].double().cpu().numpy().reshape(nb, 3, 3)
        r = self.blk_row[:nb].cpu().numpy().astype(np.int64)
        c = self.col[:nb].cpu().numpy().astype(np.int64)
        off = r != c
        r, c = np.concatenate([r, c[off]]), np.concatenate([c, r[off]])
        v = np.concatenate([v, v[off]])
        rows = np.broadcast_to((6 * r)[:, None, None] + np.arange(3)[None, :, None], v.shape)
        cols = np.broadcast_to((6 * c)[:, None, None] + np.arange(3)[None, None, :], v.shape)
        if drop_tiny:
            keep = np.abs(v) > 1e-30
            return sp.csr_matrix((v[keep], (rows[keep], cols[keep])), shape=(ndof, ndof))
        return sp.csr_matrix((v.ravel(), (rows.ravel(), cols.ravel())), shape=(ndof, ndof))
