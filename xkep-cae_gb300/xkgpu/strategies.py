"""GPU implementations of xkep-cae's Strategy surface for the assembly path.

Each class keeps the method names, argument meaning, return values, in-place
pair updates and error behaviour of the reference class it replaces, so that it
can be handed to the reference's Newton loop in place of the original:

==============================  ====================================================================
class                           replaces (reference file:line)
==============================  ====================================================================
GpuPointToPoint                 PointToPointProcess (contact/geometry/strategy.py:311-371)
GpuLineToLineGauss              LineToLineGaussProcess (contact/geometry/strategy.py:374-467)
GpuMortarSegment                MortarSegmentProcess (contact/geometry/strategy.py:470-535)
create_contact_geometry_strategy  _create_contact_geometry_strategy (contact/geometry/strategy.py:541-579)
GpuKelvinVoigtCoating           KelvinVoigtCoatingProcess (contact/coating/strategy.py:80-376)
GpuNoCoating                    NoCoatingProcess (contact/coating/strategy.py:19-77)
create_coating_strategy         _create_coating_strategy (contact/coating/strategy.py:379-400)
GpuHuberContactForce            HuberContactForceProcess (contact/contact_force/strategy.py:70-254)
GpuCoulombReturnMapping         CoulombReturnMappingProcess (contact/friction/strategy.py:48-170)
GpuDetectCandidatesProcess      DetectCandidatesProcess (contact/_manager_process.py:157-291)
GpuUpdateGeometryProcess        UpdateGeometryProcess (contact/_manager_process.py:312-408)
GpuCRBeamAssembler              ULCRBeamAssembler (elements/_beam_assembler.py:19-196)
==============================  ====================================================================

Pair lists stay in the caller's representation (frozen pair / state
dataclasses with the reference's field names).  A call packs the list into the
device pair table over a synthetic mesh of two elements per pair (element 2i
is pair i's side A, 2i+1 its side B, with the pair's own node ids and radii),
runs the kernels and writes the changed state fields back by replacing the
list items, as the reference does.  All arithmetic is in the xkgpu kernels;
the host only packs, unpacks and builds the scipy outputs.  For large models
the device-resident ``AssemblyEngine`` avoids the per-call packing.
"""

from __future__ import annotations

import ctypes as C
import dataclasses
import enum
import sys
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib as L
from .device import (DeviceBeam, DeviceContactPattern, DeviceMesh, DevicePairTable, as_dev, ptr, require_cuda,
                     stream_handle)

# ----------------------------------------------------------------------------- pair types


class ContactStatus(enum.Enum):
    """Contact status codes (``contact/_types.py:8-13``)."""

    INACTIVE = 0
    ACTIVE = 1
    SLIDING = 2


@dataclass(frozen=True)
class ContactState:
    """Per-pair state with the reference's field names (``contact/_contact_pair.py:38-66``)."""

    s: float = 0.0
    t: float = 0.0
    gap: float = 0.0
    normal: np.ndarray = field(default_factory=lambda: np.zeros(3))
    tangent1: np.ndarray = field(default_factory=lambda: np.zeros(3))
    tangent2: np.ndarray = field(default_factory=lambda: np.zeros(3))
    lambda_n: float = 0.0
    k_pen: float = 0.0
    k_t: float = 0.0
    p_n: float = 0.0
    z_t: np.ndarray = field(default_factory=lambda: np.zeros(2))
    q_trial_norm: float = 0.0
    status: ContactStatus = ContactStatus.INACTIVE
    stick: bool = True
    dissipation: float = 0.0
    coating_compression: float = 0.0
    coating_compression_prev: float = 0.0
    coating_z_t: np.ndarray = field(default_factory=lambda: np.zeros(2))
    coating_stick: bool = True
    coating_q_trial_norm: float = 0.0
    coating_dissipation: float = 0.0
    gp_z_t: list | None = None
    gp_stick: list | None = None
    gp_q_trial_norm: list | None = None


@dataclass(frozen=True)
class ContactPair:
    """Contact pair with the reference's field names (``contact/_contact_pair.py:69-81``)."""

    elem_a: int
    elem_b: int
    nodes_a: np.ndarray
    nodes_b: np.ndarray
    state: ContactState = field(default_factory=ContactState)
    radius_a: float = 0.0
    radius_b: float = 0.0
    core_radius_a: float = 0.0
    core_radius_b: float = 0.0


def pair_types():
    """(pair class, state class, status enum) for new pairs.

    Inside a process that has already loaded the reference's contact module the
    reference's own classes are used, so that its ``status == ContactStatus.X``
    comparisons keep working; otherwise the look-alike classes above.
    """
    mp = sys.modules.get("xkep_cae.contact._contact_pair")
    mt = sys.modules.get("xkep_cae.contact._types")
    if mp is not None and mt is not None:
        return mp._ContactPairOutput, mp._ContactStateOutput, mt.ContactStatus
    return ContactPair, ContactState, ContactStatus


def _code(status) -> int:
    return int(getattr(status, "value", status))


def _status_like(template, code: int):
    """``code`` as the status type that ``template`` uses (an Enum member or a plain int)."""
    if isinstance(template, enum.Enum):
        return type(template)(int(code))
    return int(code)


def _evolve(pair, **state_kw):
    return dataclasses.replace(pair, state=dataclasses.replace(pair.state, **state_kw))


def pack_pairs(pairs) -> dict:
    """Host arrays (oracle layout) of a list of pair objects."""
    n = len(pairs)
    st = [p.state for p in pairs]
    d = {"nodes": np.zeros((n, 4), np.int64)}
    if n:
        d["nodes"][:, 0:2] = np.array([np.asarray(p.nodes_a, np.int64)[:2] for p in pairs])
        d["nodes"][:, 2:4] = np.array([np.asarray(p.nodes_b, np.int64)[:2] for p in pairs])
    d["ea"] = np.array([int(p.elem_a) for p in pairs], np.int64)
    d["eb"] = np.array([int(p.elem_b) for p in pairs], np.int64)
    d["ra"] = np.array([float(p.radius_a) for p in pairs], np.float64)
    d["rb"] = np.array([float(p.radius_b) for p in pairs], np.float64)
    d["ca"] = np.array([float(getattr(p, "core_radius_a", 0.0)) for p in pairs], np.float64)
    d["cb"] = np.array([float(getattr(p, "core_radius_b", 0.0)) for p in pairs], np.float64)
    for k in ("coating_compression", "coating_compression_prev", "coating_q_trial_norm", "coating_dissipation"):
        d[k] = np.array([float(getattr(x, k, 0.0)) for x in st], np.float64)
    d["coating_z_t"] = np.array([np.asarray(getattr(x, "coating_z_t", np.zeros(2)), np.float64).reshape(2)
                                 for x in st]).reshape(n, 2)
    d["coating_stick"] = np.array([bool(getattr(x, "coating_stick", True)) for x in st], bool)
    for k in ("s", "t", "gap", "lambda_n", "k_pen", "k_t", "p_n", "q_trial_norm", "dissipation"):
        d[k] = np.array([float(getattr(x, k)) for x in st], np.float64)
    for k, src, w in (("normal", "normal", 3), ("t1", "tangent1", 3), ("t2", "tangent2", 3), ("z_t", "z_t", 2)):
        d[k] = np.array([np.asarray(getattr(x, src), np.float64).reshape(w) for x in st]).reshape(n, w)
    d["status"] = np.array([_code(x.status) for x in st], np.int8)
    d["stick"] = np.array([bool(x.stick) for x in st], bool)
    return d


class PairBatch:
    """A pair list (or an oracle-layout table) on the device.

    The mesh is synthetic: two elements per pair holding the pair's node ids and
    radii, so the element-indexed kernels see exactly the pair's data.  ``coords``
    are the node positions used by the narrowphase (zeros when only the pair
    state is read).
    """

    def __init__(self, pairs, n_nodes: int, *, coords=None, device=None, core: bool = False,
                 all_members: bool = False):
        """``core``: the synthetic elements carry the pairs' core radii (the coating geometry);
        ``all_members``: every pair is a member of the contact pattern (the coating forces)."""
        self.host = pairs if isinstance(pairs, dict) else pack_pairs(pairs)
        h = self.host
        n = int(h["ea"].shape[0])
        self.n = n
        dev = require_cuda(device)
        nodes = np.asarray(h["nodes"], np.int64).reshape(n, 4)
        conn = np.empty((2 * n, 2), np.int64)
        conn[0::2], conn[1::2] = nodes[:, 0:2], nodes[:, 2:4]
        radii = np.empty(2 * n, np.float64)
        radii[0::2], radii[1::2] = (h["ca"], h["cb"]) if core else (h["ra"], h["rb"])
        X = np.zeros((n_nodes, 3)) if coords is None else np.asarray(coords, np.float64).reshape(-1, 3)
        if X.shape[0] < n_nodes:
            X = np.concatenate([X, np.zeros((n_nodes - X.shape[0], 3))])
        self.mesh = DeviceMesh(X, conn, radii, device=dev)
        self.table = DevicePairTable(dev, cap=max(n, 16))
        d = {k: h[k] for k in ("s", "t", "gap", "normal", "t1", "t2", "lambda_n", "k_pen", "k_t", "p_n", "z_t",
                               "q_trial_norm", "dissipation", "status", "stick")}
        d["ea"] = np.arange(0, 2 * n, 2, dtype=np.int64)
        d["eb"] = np.arange(1, 2 * n, 2, dtype=np.int64)
        if all_members:
            d["status"] = np.ones(n, np.int8)
        self.table.from_host(d, 2 * n)
        self.u0 = torch.zeros(self.mesh.ndof, dtype=torch.float64, device=dev)
        self.pattern = None
        self.rec = None
        self.coat = None

    @property
    def device(self):
        return self.mesh.device

    def build_pattern(self):
        self.pattern = DeviceContactPattern(self.mesh)
        self.pattern.build(self.table)
        self.rec = torch.zeros(L.REC_STRIDE[L.XK_OUT_SPLIT] * max(self.pattern.cap_members, 1),
                               dtype=torch.float64, device=self.device)

    def step(self, stages: int, cp, u=None, u_ref=None):
        """Run the selected pair stages over the members (split records)."""
        if self.pattern is None:
            self.build_pattern()
        uu = self.u0 if u is None else u
        L.call("xk_pair_step", C.byref(self.mesh.c), C.byref(self.table.c), C.byref(self.pattern.c), ptr(uu),
               ptr(u_ref), C.byref(cp), stages, L.XK_FP64, L.XK_OUT_SPLIT, ptr(self.rec), stream_handle())

    def force(self, which: int, ndof: int) -> np.ndarray:
        """sum_k c_k v over the members' split records (the reference's raw f_n or f_f)."""
        out = torch.zeros(self.mesh.ndof, dtype=torch.float64, device=self.device)
        L.call("xk_contact_gather_force", C.byref(self.pattern.c), ptr(self.rec), L.XK_FP64, L.XK_OUT_SPLIT, which,
               None, 1.0, None, None, ptr(out), None, stream_handle())
        f = np.zeros(ndof)
        f[: min(ndof, out.numel())] = out.cpu().numpy()[:ndof]
        return f

    def tangent(self, which: int, ndof: int) -> sp.csr_matrix:
        """sum c_k c_l B over the members as an ndof x ndof CSR; |value| <= 1e-30 dropped as in the reference."""
        nb = self.pattern.nnzb
        if nb == 0:
            return sp.csr_matrix((ndof, ndof))
        K = torch.zeros(9 * nb, dtype=torch.float64, device=self.device)
        L.call("xk_contact_gather_tangent", C.byref(self.pattern.c), ptr(self.rec), L.XK_FP64, L.XK_OUT_SPLIT,
               which, L.XK_GATHER_DEFAULT, ptr(K), stream_handle())
        return self.pattern.to_csr(K, ndof, drop_tiny=True)

    def narrowphase(self, cp, update_active: bool):
        L.call("xk_narrowphase", C.byref(self.mesh.c), C.byref(self.table.c), ptr(self.u0), C.byref(cp),
               int(update_active), stream_handle())

    def state(self) -> dict:
        return self.table.to_host()

    # -- coating -------------------------------------------------------------
    def coating_state(self):
        """Device copy of the pairs' coating state (``xk_coating_state``)."""
        if self.coat is None:
            h, dev = self.host, self.device
            t = {"cc": h["coating_compression"], "cc_prev": h["coating_compression_prev"],
                 "z_t": np.ascontiguousarray(h["coating_z_t"].T).ravel(), "q_trial_norm": h["coating_q_trial_norm"],
                 "dissipation": h["coating_dissipation"]}
            self.coat_t = {k: as_dev(np.asarray(v, np.float64), torch.float64, dev) for k, v in t.items()}
            self.coat_t["stick"] = as_dev(h["coating_stick"].astype(np.uint8), torch.uint8, dev)
            self.coat = L.CoatingState(*(ptr(self.coat_t[k]) for k in ("cc", "cc_prev", "z_t", "stick",
                                                                         "q_trial_norm", "dissipation")))
        return self.coat

    def coating_geometry(self, cp, coat_total: np.ndarray, update_active: bool) -> np.ndarray:
        """Narrowphase on the core radii, then the coating compression (and the active set)."""
        self.narrowphase(cp, False)
        ct = as_dev(np.asarray(coat_total, np.float64), torch.float64, self.device)
        cc = torch.zeros(max(self.n, 1), dtype=torch.float64, device=self.device)
        L.call("xk_coating_geometry", C.byref(self.table.c), ptr(ct), C.byref(cp), int(update_active), ptr(cc),
               stream_handle())
        return cc[: self.n].cpu().numpy()

    def coating_step(self, stages: int, params, u=None, u_ref=None):
        if self.pattern is None:
            self.build_pattern()
        L.call("xk_coating_step", C.byref(self.table.c), C.byref(self.pattern.c), C.byref(self.coating_state()),
               ptr(u), ptr(u_ref), C.byref(params), int(stages), ptr(self.rec), stream_handle())

    def member_pairs(self) -> np.ndarray:
        """Pair index of every member (record order)."""
        return self.pattern.members[: self.pattern.n_members].cpu().numpy().astype(np.int64)


def _contact_params(k_pen=0.0, k_t_ratio=0.0, mu_eff=0.0, smoothing_delta=0.0, g_on=0.0, g_off=0.0,
                    allow_deactivation=True):
    return L.ContactParams(float(k_pen), float(k_t_ratio), float(mu_eff), float(smoothing_delta), float(g_on),
                           float(g_off), int(bool(allow_deactivation)))


def _check_dofs(ndof_per_node: int):
    if int(ndof_per_node) != 6:
        raise ValueError(f"the GPU contact path uses 6 DOFs per node (ux,uy,uz,θx,θy,θz), got {ndof_per_node}")


def _n_nodes(ndof: int, ndof_per_node: int = 6) -> int:
    return max(int(ndof) // int(ndof_per_node), 0)


def _dev_vec(x, device) -> torch.Tensor | None:
    return None if x is None else as_dev(np.asarray(x, dtype=np.float64).ravel(), torch.float64, device)


# ----------------------------------------------------------------------------- geometry


def _write_geometry(pairs, st: dict, idx, with_status: bool, cc=None):
    for i in idx:
        kw = {"s": float(st["s"][i]), "t": float(st["t"][i]), "gap": float(st["gap"][i]),
              "normal": st["normal"][i].copy(), "tangent1": st["t1"][i].copy(), "tangent2": st["t2"][i].copy()}
        if with_status:
            kw["status"] = _status_like(pairs[i].state.status, st["status"][i])
        if cc is not None:
            kw["coating_compression"] = float(cc[i])
        pairs[i] = _evolve(pairs[i], **kw)


def _coated_geometry(pairs, coords, cp, update_active: bool, device):
    """The coating branch of the geometry update (``_manager_process.py:351-360,386-396``,
    ``geometry/strategy.py:242-254``): the narrowphase on the core radii, gap = dist - (core_a + core_b),
    coating_compression = max(0, coat_total - gap) and the hysteresis with the coating term."""
    batch = PairBatch(pairs, coords.shape[0], coords=coords, device=device, core=True)
    h = batch.host
    coat_total = (h["ra"] - h["ca"]) + (h["rb"] - h["cb"])
    cc = batch.coating_geometry(cp, coat_total, update_active)
    _write_geometry(pairs, batch.state(), range(len(pairs)), update_active, cc)


class GpuPointToPoint:
    """``PointToPointProcess`` (``contact/geometry/strategy.py:311-371``) on the GPU.

    ``detect`` is the AABB broadphase with shared-node exclusion (when
    ``exclude_same_layer``, the reference's name for it) and the initial
    narrowphase with g_on = g_off = 0 (``strategy.py:135-202``);
    ``update_geometry`` the narrowphase with the active-set hysteresis
    (``strategy.py:205-308``); ``build_constraint_jacobian`` the PtP Jacobian
    (``strategy.py:83-132``).
    """

    def __init__(self, *, exclude_same_layer: bool = True, device=None) -> None:
        self._exclude_same_layer = exclude_same_layer
        self._device = device

    def detect(self, node_coords, connectivity, radii) -> list:
        coords = np.asarray(node_coords, dtype=float)
        conn = np.asarray(connectivity, dtype=np.int64).reshape(-1, 2)
        ne = conn.shape[0]
        if ne < 2:
            return []
        r = np.full(ne, float(radii)) if np.isscalar(radii) else np.asarray(radii, dtype=float)
        mesh = DeviceMesh(coords, conn, r, device=self._device)
        bp = L.BPParams(0.0, int(bool(self._exclude_same_layer)), 0, 0, 0.0)
        cands = _broadphase(mesh, bp, mesh.device)
        table = _merge(mesh, DevicePairTable(mesh.device, cap=16), cands)
        u0 = torch.zeros(mesh.ndof, dtype=torch.float64, device=mesh.device)
        L.call("xk_narrowphase", C.byref(mesh.c), C.byref(table.c), ptr(u0), C.byref(_contact_params()), 1,
               stream_handle())
        st = table.to_host()
        Pair, State, Status = pair_types()
        out = []
        for i in range(table.n):
            a, b = int(st["ea"][i]), int(st["eb"][i])
            state = State(s=float(st["s"][i]), t=float(st["t"][i]), gap=float(st["gap"][i]),
                          normal=st["normal"][i].copy(), tangent1=st["t1"][i].copy(), tangent2=st["t2"][i].copy(),
                          status=Status(int(st["status"][i])))
            out.append(Pair(elem_a=a, elem_b=b, nodes_a=conn[a].copy(), nodes_b=conn[b].copy(), state=state,
                            radius_a=float(r[a]), radius_b=float(r[b])))
        return out

    def compute_gap(self, pair, node_coords) -> float:
        if hasattr(pair, "state") and hasattr(pair.state, "gap"):
            return float(pair.state.gap)
        return 0.0

    def update_geometry(self, pairs: list, node_coords, *, config=None) -> None:
        if not pairs:
            return
        coords = np.asarray(node_coords, dtype=float).reshape(-1, 3)
        g_on = getattr(config, "g_on", 0.0) if config is not None else 0.0
        g_off = getattr(config, "g_off", 0.0) if config is not None else 0.0
        if config is not None and getattr(config, "coating_stiffness", 0.0) > 0.0:
            _coated_geometry(pairs, coords, _contact_params(g_on=g_on, g_off=g_off, allow_deactivation=True), True,
                             self._device)
            return
        batch = PairBatch(pairs, coords.shape[0], coords=coords, device=self._device)
        batch.narrowphase(_contact_params(g_on=g_on, g_off=g_off, allow_deactivation=True), True)
        _write_geometry(pairs, batch.state(), range(len(pairs)), True)

    def build_constraint_jacobian(self, pairs: list, ndof_total: int, ndof_per_node: int = 6):
        _check_dofs(ndof_per_node)
        active_idx = [i for i, p in enumerate(pairs) if _code(p.state.status) != 0]
        if not active_idx:
            return sp.csr_matrix((0, ndof_total)), []
        batch = PairBatch(pairs, _n_nodes(ndof_total), device=self._device)
        return _jacobian(batch, ndof_total)


def pair_gauss_points(pairs: list, node_coords, *, default: int = 3, device=None) -> np.ndarray:
    """Gauss-point count of every pair at ``node_coords`` (``_auto_select_n_gauss``,
    ``contact/geometry/_compute.py:264-291``), computed on the GPU."""
    if not pairs:
        return np.zeros(0, dtype=np.int64)
    coords = np.asarray(node_coords, dtype=float).reshape(-1, 3)
    batch = PairBatch(pairs, coords.shape[0], coords=coords, device=device)
    out = torch.empty(batch.n, dtype=torch.int8, device=batch.device)
    L.call("xk_pair_gauss_points", C.byref(batch.mesh.c), C.byref(batch.table.c), None, int(default), ptr(out),
           stream_handle())
    return out.cpu().numpy().astype(np.int64)


class GpuLineToLineGauss(GpuPointToPoint):
    """``LineToLineGaussProcess`` (``contact/geometry/strategy.py:374-467``) on the GPU.

    The reference evaluates this strategy's geometry exactly as the
    point-to-point one (``_batch_update_geometry``) and, with ``auto_gauss``,
    then stores the angle-based Gauss-point count in each pair that has an
    ``_n_gauss`` attribute (``strategy.py:436-451``); the constraint Jacobian is
    the point-to-point one.  So is this class's.
    """

    def __init__(self, *, n_gauss: int = 2, exclude_same_layer: bool = True, auto_gauss: bool = False,
                 device=None) -> None:
        super().__init__(exclude_same_layer=exclude_same_layer, device=device)
        self._n_gauss = n_gauss
        self._auto_gauss = auto_gauss

    def update_geometry(self, pairs: list, node_coords, *, config=None) -> None:
        super().update_geometry(pairs, node_coords, config=config)
        if self._auto_gauss and len(pairs) > 0:
            n_gp = pair_gauss_points(pairs, node_coords, device=self._device)
            for pair, n in zip(pairs, n_gp):
                if hasattr(pair, "_n_gauss"):
                    pair._n_gauss = int(n)


class GpuMortarSegment(GpuPointToPoint):
    """``MortarSegmentProcess`` (``contact/geometry/strategy.py:470-535``) on the GPU: the
    point-to-point geometry and Jacobian, as in the reference."""

    def __init__(self, *, n_gauss: int = 2, exclude_same_layer: bool = True, device=None) -> None:
        super().__init__(exclude_same_layer=exclude_same_layer, device=device)
        self._n_gauss = n_gauss


def create_contact_geometry_strategy(*, mode: str = "point_to_point", exclude_same_layer: bool = True,
                                     n_gauss: int = 2, auto_gauss: bool = False, line_contact: bool = False,
                                     use_mortar: bool = False, device=None):
    """``_create_contact_geometry_strategy`` (``contact/geometry/strategy.py:541-579``): the same
    mode selection (``use_mortar`` over ``line_contact`` over ``mode``) with the GPU classes."""
    if use_mortar:
        mode = "mortar"
    elif line_contact:
        mode = "line_to_line"
    if mode == "mortar":
        return GpuMortarSegment(n_gauss=n_gauss, exclude_same_layer=exclude_same_layer, device=device)
    if mode == "line_to_line":
        return GpuLineToLineGauss(n_gauss=n_gauss, exclude_same_layer=exclude_same_layer, auto_gauss=auto_gauss,
                                  device=device)
    return GpuPointToPoint(exclude_same_layer=exclude_same_layer, device=device)


def _jacobian(batch: PairBatch, ndof: int):
    n = batch.n
    dev = batch.device
    rows = torch.empty(12 * n, dtype=torch.int32, device=dev)
    cols = torch.empty(12 * n, dtype=torch.int32, device=dev)
    vals = torch.empty(12 * n, dtype=torch.float64, device=dev)
    pidx = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    n_rows = C.c_int64(0)
    L.call("xk_constraint_jacobian", C.byref(batch.mesh.c), C.byref(batch.table.c), ptr(rows), ptr(cols), ptr(vals),
           ptr(pidx), n, C.byref(n_rows), stream_handle())
    m = int(n_rows.value)
    r = rows[: 12 * m].cpu().numpy()
    c = cols[: 12 * m].cpu().numpy()
    v = vals[: 12 * m].cpu().numpy()
    keep = np.abs(v) > 1e-30
    G = sp.coo_matrix((v[keep], (r[keep], c[keep])), shape=(m, ndof)).tocsr()
    return G, [int(i) for i in pidx[:m].cpu().numpy()]


def _broadphase(mesh: DeviceMesh, bp, device) -> torch.Tensor:
    u0 = torch.zeros(mesh.ndof, dtype=torch.float64, device=device)
    cands = torch.zeros(2 * max(4 * mesh.n_elems, 1024), dtype=torch.int32, device=device)
    n_out, n_raw, n_pre = C.c_int64(0), C.c_int64(0), C.c_int64(0)
    for _ in range(3):
        code = L.call("xk_broadphase", C.byref(mesh.c), ptr(u0), C.byref(bp), ptr(cands), cands.numel() // 2,
                      C.byref(n_out), C.byref(n_raw), C.byref(n_pre), stream_handle(), allow=(L.XK_ERR_CAPACITY,))
        if code == L.XK_OK:
            return cands[: 2 * int(n_out.value)]
        cands = torch.zeros(2 * int(n_out.value * 1.25 + 1024), dtype=torch.int32, device=device)
    raise RuntimeError("broadphase candidate capacity did not converge")


def _merge(mesh: DeviceMesh, old: DevicePairTable, cands: torch.Tensor) -> DevicePairTable:
    nc = cands.numel() // 2
    out = DevicePairTable(mesh.device, cap=max(old.n + nc, 16))
    L.call("xk_pairs_merge", C.byref(mesh.c), C.byref(old.c), ptr(cands), nc, C.byref(out.c), stream_handle())
    out.set_n(out.c.n)
    return out


# ----------------------------------------------------------------------------- normal force


class GpuHuberContactForce:
    """``HuberContactForceProcess`` (``contact/contact_force/strategy.py:70-254``) on the GPU.

    ``evaluate(u, manager, k_pen)`` returns ``(f_c, residuals)`` with
    f_c = sum p_n c_k n over the non-INACTIVE pairs of ``manager.pairs`` and
    writes each such pair's ``state.p_n``; ``tangent(u, manager, k_pen)``
    returns K_mat - K_geo as an ndof x ndof CSR.
    """

    def __init__(self, ndof: int, ndof_per_node: int = 6, *, smoothing_delta: float = 0.0, device=None) -> None:
        _check_dofs(ndof_per_node)
        self._ndof = int(ndof)
        self._ndof_per_node = ndof_per_node
        self._smoothing_delta = smoothing_delta
        self._device = device

    def evaluate(self, u, manager, k_pen: float):
        pairs = getattr(manager, "pairs", None)
        if not pairs:
            return np.zeros(self._ndof), np.zeros(0)
        batch = PairBatch(pairs, _n_nodes(self._ndof), device=self._device)
        batch.step(L.XK_STAGE_NORMAL, _contact_params(k_pen=k_pen, smoothing_delta=self._smoothing_delta))
        f = batch.force(L.XK_WHICH_NORMAL, self._ndof)
        st = batch.state()
        live = np.nonzero(st["status"] != 0)[0]
        for i in live:
            pairs[i] = _evolve(pairs[i], p_n=float(st["p_n"][i]))
        p_n, gap = st["p_n"][live], st["gap"][live]
        residuals = np.where(p_n > 0.0, k_pen * gap, 0.0)
        return f, residuals

    def tangent(self, u, manager, k_pen: float) -> sp.csr_matrix:
        pairs = getattr(manager, "pairs", None)
        if not pairs:
            return sp.csr_matrix((self._ndof, self._ndof))
        batch = PairBatch(pairs, _n_nodes(self._ndof), device=self._device)
        batch.step(L.XK_STAGE_TANGENT, _contact_params(k_pen=k_pen, smoothing_delta=self._smoothing_delta))
        return batch.tangent(L.XK_WHICH_NORMAL, self._ndof)


def smooth_normal_force(gaps, k_pen: float, lambdas=None, *, delta: float = 1e-4, device=None):
    """``_evaluate_smooth_normal_force_vectorized`` (``contact/penalty/law_normal.py:129-149``) on the GPU.

    Returns ``(p_n, dp_dg)`` as NumPy arrays (or device tensors for device input).
    """
    dev = require_cuda(device)
    on_dev = isinstance(gaps, torch.Tensor) and gaps.is_cuda
    g = _dev_vec(gaps, dev) if not on_dev else gaps.to(torch.float64).contiguous()
    lam = None if lambdas is None else (_dev_vec(lambdas, dev) if not on_dev else lambdas.to(torch.float64))
    p = torch.empty_like(g)
    dp = torch.empty_like(g)
    L.call("xk_softplus_normal_law", g.numel(), ptr(g), ptr(lam), float(k_pen), float(delta), ptr(p), ptr(dp),
           stream_handle())
    return (p, dp) if on_dev else (p.cpu().numpy(), dp.cpu().numpy())


# ----------------------------------------------------------------------------- friction


def mu_effective(mu: float, ramp_counter: int, ramp_steps: int) -> float:
    """mu * min(1, counter / ramp_steps), or mu without a ramp (``friction/law_friction.py:183-195``)."""
    if ramp_steps <= 0:
        return mu
    return mu * min(1.0, ramp_counter / ramp_steps)


def friction_tangent_2x2(k_t, p_n, mu, z_t, q_trial_norm, stick) -> np.ndarray:
    """Consistent 2x2 tangent of the Coulomb return mapping (``friction/law_friction.py:126-153``)."""
    if stick:
        return k_t * np.eye(2)
    qn = float(np.linalg.norm(z_t))
    if q_trial_norm < 1e-30 or qn < 1e-30:
        return k_t * np.eye(2)
    qh = np.asarray(z_t, dtype=float) / qn
    return (mu * p_n / q_trial_norm) * k_t * (np.eye(2) - np.outer(qh, qh))


class GpuCoulombReturnMapping:
    """``CoulombReturnMappingProcess`` (``contact/friction/strategy.py:48-170``) on the GPU.

    ``evaluate(u, contact_pairs, mu, u_ref=...)`` runs the return mapping of
    every pair with p_n > 0 (``friction/_assembly.py:260-342``), updates those
    pairs' state in the list and returns ``(f_friction, residual)``;
    ``tangent`` returns K_mat + K_geo of the friction part.  The extra members
    the reference's solver uses (``friction_tangents``, ``compute_k_t``,
    ``compute_mu_effective``, ``set_k_pen``, ``set_k_t_ratio``,
    ``set_mu_ramp_counter``) are provided.
    """

    def __init__(self, ndof: int, ndof_per_node: int = 6, *, k_pen: float = 0.0, k_t_ratio: float = 1.0,
                 mu_ramp_counter: int = 0, mu_ramp_steps: int = 0, device=None) -> None:
        _check_dofs(ndof_per_node)
        self._ndof = int(ndof)
        self._ndof_per_node = ndof_per_node
        self._k_pen = k_pen
        self._k_t_ratio = k_t_ratio
        self._mu_ramp_counter = mu_ramp_counter
        self._mu_ramp_steps = mu_ramp_steps
        self._friction_tangents: dict[int, np.ndarray] = {}
        self._friction_forces_local: dict[int, np.ndarray] = {}
        self._device = device

    @property
    def friction_tangents(self) -> dict:
        return self._friction_tangents

    def compute_k_t(self) -> float:
        return self._k_pen * self._k_t_ratio

    def compute_mu_effective(self, mu: float) -> float:
        return mu_effective(mu, self._mu_ramp_counter, self._mu_ramp_steps)

    def set_k_pen(self, k_pen: float) -> None:
        self._k_pen = k_pen

    def set_k_t_ratio(self, k_t_ratio: float) -> None:
        self._k_t_ratio = k_t_ratio

    def set_mu_ramp_counter(self, counter: int) -> None:
        self._mu_ramp_counter = counter

    def _params(self, mu_eff):
        return _contact_params(k_pen=self._k_pen, k_t_ratio=self._k_t_ratio, mu_eff=mu_eff)

    def evaluate(self, u, contact_pairs: list, mu: float, **kwargs):
        self._friction_tangents, self._friction_forces_local = {}, {}
        if not contact_pairs:
            return np.zeros(self._ndof), np.zeros(0)
        mu_eff = self.compute_mu_effective(mu)
        batch = PairBatch(contact_pairs, _n_nodes(self._ndof), device=self._device)
        dev = batch.device
        u_d = _dev_vec(u, dev)
        u_ref = kwargs.get("u_ref")
        ur_d = _dev_vec(u_ref, dev) if u_ref is not None else None
        batch.step(L.XK_STAGE_FRICTION, self._params(mu_eff), u_d, ur_d)
        f = batch.force(L.XK_WHICH_FRICTION, self._ndof)
        st = batch.state()
        done = np.nonzero((batch.host["p_n"] > 0.0) & (mu_eff > 0.0))[0]
        residuals = []
        for i in done:
            q = st["z_t"][i].copy()
            contact_pairs[i] = _evolve(contact_pairs[i], k_pen=float(st["k_pen"][i]), k_t=float(st["k_t"][i]),
                                       z_t=q, stick=bool(st["stick"][i]), q_trial_norm=float(st["q_trial_norm"][i]),
                                       dissipation=float(st["dissipation"][i]),
                                       status=_status_like(contact_pairs[i].state.status, st["status"][i]))
            qn = float(np.linalg.norm(q))
            if qn < 1e-30:
                continue
            residuals.append(max(0.0, qn - mu_eff * float(st["p_n"][i])))
            self._friction_forces_local[int(i)] = q
            self._friction_tangents[int(i)] = friction_tangent_2x2(
                float(st["k_t"][i]), float(st["p_n"][i]), mu_eff, q, float(st["q_trial_norm"][i]),
                bool(st["stick"][i]))
        return f, (np.array(residuals) if residuals else np.zeros(0))

    def tangent(self, u, contact_pairs: list, mu: float, **kwargs) -> sp.csr_matrix:
        if not contact_pairs or not self._friction_forces_local:
            return sp.csr_matrix((self._ndof, self._ndof))
        mu_eff = self.compute_mu_effective(mu)
        batch = PairBatch(contact_pairs, _n_nodes(self._ndof), device=self._device)
        batch.step(L.XK_STAGE_TANGENT, self._params(mu_eff))
        return batch.tangent(L.XK_WHICH_FRICTION, self._ndof)


# ----------------------------------------------------------------------------- manager processes


# ----------------------------------------------------------------------------- coating


def _coating_params(config, dt: float = 0.0):
    return L.CoatingParams(float(getattr(config, "coating_stiffness", 0.0)),
                           float(getattr(config, "coating_damping", 0.0)), float(getattr(config, "coating_mu", 0.0)),
                           float(getattr(config, "coating_k_t_ratio", 0.5)), float(dt))


def _coating_batch(pairs, node_coords, ndof_per_node, device):
    _check_dofs(ndof_per_node)
    n_nodes = np.asarray(node_coords, dtype=float).reshape(-1, 3).shape[0]
    return PairBatch(pairs, n_nodes, device=device, all_members=True), n_nodes


class GpuNoCoating:
    """``NoCoatingProcess`` (``contact/coating/strategy.py:19-77``): zero forces and stiffness."""

    def forces(self, pairs: list, node_coords, config, dt: float) -> np.ndarray:
        return np.zeros(len(node_coords) * getattr(config, "ndof_per_node", 6))

    def stiffness(self, pairs: list, node_coords, config, ndof_total: int, dt: float) -> sp.csr_matrix:
        return sp.csr_matrix((ndof_total, ndof_total))

    def friction_forces(self, pairs: list, node_coords, config, u_cur, u_ref) -> np.ndarray:
        return np.zeros_like(u_cur)

    def friction_stiffness(self, pairs: list, node_coords, config, ndof_total: int) -> sp.csr_matrix:
        return sp.csr_matrix((ndof_total, ndof_total))

    def process(self, input_data=None):
        return None


class GpuKelvinVoigtCoating:
    """``KelvinVoigtCoatingProcess`` (``contact/coating/strategy.py:80-400``) on the GPU.

    The coating between two wire cores acts as a spring k and a dashpot c on
    the coating compression cc (state ``coating_compression``, set by the
    coating branch of the geometry update), with Coulomb friction on the
    coating surface (tangential penalty k * coating_k_t_ratio, friction
    coefficient coating_mu).  Each method packs the pair list, runs the
    coating stage of ``xk_coating_step`` over every pair and gathers the
    records; ``friction_forces`` writes the updated coating friction state back
    into ``pairs`` as the reference does.
    """

    def __init__(self, device=None) -> None:
        self._device = device

    def forces(self, pairs: list, node_coords, config, dt: float) -> np.ndarray:
        ndpn = getattr(config, "ndof_per_node", 6)
        n_nodes = np.asarray(node_coords, dtype=float).reshape(-1, 3).shape[0]
        if not pairs:
            return np.zeros(n_nodes * ndpn)
        batch, _ = _coating_batch(pairs, node_coords, ndpn, self._device)
        batch.coating_step(L.XK_COAT_FORCE, _coating_params(config, dt))
        return batch.force(L.XK_WHICH_NORMAL, n_nodes * ndpn)

    def stiffness(self, pairs: list, node_coords, config, ndof_total: int, dt: float) -> sp.csr_matrix:
        if not pairs:
            return sp.csr_matrix((ndof_total, ndof_total))
        batch, _ = _coating_batch(pairs, node_coords, getattr(config, "ndof_per_node", 6), self._device)
        batch.coating_step(L.XK_COAT_TANGENT, _coating_params(config, dt))
        return batch.tangent(L.XK_WHICH_NORMAL, ndof_total)

    def friction_forces(self, pairs: list, node_coords, config, u_cur, u_ref) -> np.ndarray:
        u_cur = np.asarray(u_cur, dtype=float)
        if getattr(config, "coating_mu", 0.0) <= 0.0 or not pairs:
            return np.zeros_like(u_cur)
        batch, _ = _coating_batch(pairs, node_coords, getattr(config, "ndof_per_node", 6), self._device)
        dev = batch.device
        u = as_dev(u_cur.ravel(), torch.float64, dev)
        ur = as_dev(np.asarray(u_ref, dtype=float).ravel(), torch.float64, dev)
        batch.coating_step(L.XK_COAT_FRICTION, _coating_params(config), u, ur)
        f = batch.force(L.XK_WHICH_FRICTION, u_cur.size)
        t = batch.coat_t
        z = t["z_t"].view(2, -1).cpu().numpy()
        stick = t["stick"].cpu().numpy()
        qtn = t["q_trial_norm"].cpu().numpy()
        diss = t["dissipation"].cpu().numpy()
        for i in range(len(pairs)):
            pairs[i] = _evolve(pairs[i], coating_z_t=np.array([z[0, i], z[1, i]]), coating_stick=bool(stick[i]),
                               coating_q_trial_norm=float(qtn[i]), coating_dissipation=float(diss[i]))
        return f.reshape(u_cur.shape)

    def friction_stiffness(self, pairs: list, node_coords, config, ndof_total: int) -> sp.csr_matrix:
        if getattr(config, "coating_mu", 0.0) <= 0.0 or not pairs:
            return sp.csr_matrix((ndof_total, ndof_total))
        batch, _ = _coating_batch(pairs, node_coords, getattr(config, "ndof_per_node", 6), self._device)
        batch.coating_step(L.XK_COAT_FRICTION_TANGENT, _coating_params(config))
        return batch.tangent(L.XK_WHICH_FRICTION, ndof_total)

    def process(self, input_data=None):
        return None


def create_coating_strategy(*, coating_stiffness: float = 0.0, device=None):
    """``_create_coating_strategy`` (``contact/coating/strategy.py:385-400``)."""
    if coating_stiffness <= 0.0:
        return GpuNoCoating()
    return GpuKelvinVoigtCoating(device=device)


@dataclass(frozen=True)
class ContactConfig:
    """The contact settings the assembly path reads, with the reference's names and defaults
    (``_ContactConfigInput``, ``contact/_contact_pair.py:84-170``)."""

    k_t_ratio: float = 0.5
    mu: float = 0.3
    g_on: float = 0.0
    g_off: float = 1e-6
    mu_ramp_steps: int = 0
    elem_layer_map: dict | None = None
    exclude_same_layer: bool = False
    midpoint_prescreening: bool = True
    prescreening_margin: float = 0.0
    coating_stiffness: float = 0.0
    coating_damping: float = 0.0
    coating_mu: float = 0.0
    coating_k_t_ratio: float = 0.5
    smoothing_delta: float = 0.0


@dataclass(frozen=True)
class ContactManager:
    """Pair list and settings (``_ContactManagerInput``, ``contact/_contact_pair.py:173-181``)."""

    pairs: list = field(default_factory=list)
    config: ContactConfig = field(default_factory=ContactConfig)


@dataclass(frozen=True)
class DetectCandidatesInput:
    """Fields of the reference's ``DetectCandidatesInput`` (``contact/_manager_process.py:135-145``)."""

    manager: object
    node_coords: np.ndarray
    connectivity: np.ndarray
    radii: object = 0.0
    margin: float = 0.0
    cell_size: float | None = None
    core_radii: object = None


@dataclass(frozen=True)
class UpdateGeometryInput:
    """Fields of the reference's ``UpdateGeometryInput`` (``contact/_manager_process.py:294-301``)."""

    manager: object
    node_coords: np.ndarray
    allow_deactivation: bool = True
    freeze_active_set: bool = False


@dataclass(frozen=True)
class DetectCandidatesResult:
    """Output of ``GpuDetectCandidatesProcess`` (fields of ``DetectCandidatesOutput``)."""

    manager: object
    candidates: list
    n_pairs: int


@dataclass(frozen=True)
class UpdateGeometryResult:
    """Output of ``GpuUpdateGeometryProcess`` (fields of ``UpdateGeometryOutput``)."""

    manager: object
    n_active: int


def _replace_pairs(manager, pairs):
    if dataclasses.is_dataclass(manager):
        return dataclasses.replace(manager, pairs=pairs)
    new = type(manager).__new__(type(manager))
    new.__dict__.update(manager.__dict__)
    new.pairs = pairs
    return new


def _elem_layers(config, n_elems: int):
    lm = getattr(config, "elem_layer_map", None)
    if not (getattr(config, "exclude_same_layer", False) and lm is not None):
        return None
    layer = np.full(n_elems, -1, dtype=np.int64)
    for e, l in lm.items():
        if 0 <= int(e) < n_elems:
            layer[int(e)] = int(l)
    return layer


class GpuDetectCandidatesProcess:
    """``DetectCandidatesProcess`` (``contact/_manager_process.py:157-291``) on the GPU.

    ``process(inp)`` takes an object with the fields of ``DetectCandidatesInput``
    (manager, node_coords, connectivity, radii, margin, cell_size, core_radii):
    broadphase, shared-node and same-layer exclusion, midpoint prescreen
    (``config.midpoint_prescreening``), then the pair-list merge: existing pairs
    that are not candidates become INACTIVE, new candidates are appended with a
    fresh state.  The cell size does not change the candidate set.
    """

    def __init__(self, device=None) -> None:
        self._device = device

    def process(self, inp) -> DetectCandidatesResult:
        manager = inp.manager
        config = manager.config
        conn = np.asarray(inp.connectivity, dtype=np.int64).reshape(-1, 2)
        coords = np.asarray(inp.node_coords, dtype=float)
        ne = conn.shape[0]
        r = np.full(ne, float(inp.radii)) if np.isscalar(inp.radii) else np.asarray(inp.radii, dtype=float)
        cr_in = getattr(inp, "core_radii", None)
        cr = r.copy() if cr_in is None else (np.full(ne, float(cr_in)) if np.isscalar(cr_in)
                                              else np.asarray(cr_in, dtype=float))
        layer = _elem_layers(config, ne)
        mesh = DeviceMesh(coords, conn, r, layer=layer, device=self._device)
        bp = L.BPParams(float(getattr(inp, "margin", 0.0)), 1, int(layer is not None),
                        int(bool(getattr(config, "midpoint_prescreening", True))),
                        float(getattr(config, "prescreening_margin", 0.0)),
                        float(getattr(inp, "cell_size", None) or 0.0))
        cands = _broadphase(mesh, bp, mesh.device)
        old_pairs = list(manager.pairs)
        old = DevicePairTable(mesh.device, cap=max(len(old_pairs), 16))
        if old_pairs:
            h = pack_pairs(old_pairs)
            a, b = np.minimum(h["ea"], h["eb"]), np.maximum(h["ea"], h["eb"])
            h["ea"], h["eb"] = a, b
            old.from_host(h, ne)
        new = _merge(mesh, old, cands)
        st = new.to_host()  # union of old pairs and candidates, sorted by (elem_a, elem_b)
        pairs = list(old_pairs)
        old_at = {}
        for i, p in enumerate(old_pairs):
            old_at[(min(int(p.elem_a), int(p.elem_b)), max(int(p.elem_a), int(p.elem_b)))] = i
        fresh = []
        for j in range(new.n):
            key = (int(st["ea"][j]), int(st["eb"][j]))
            i = old_at.get(key)
            if i is None:
                fresh.append(j)
            elif st["status"][j] == 0 and _code(pairs[i].state.status) != 0:
                pairs[i] = _evolve(pairs[i], status=_status_like(pairs[i].state.status, 0))
        if old_pairs:  # new pairs take the classes of the caller's pairs
            Pair, State = type(old_pairs[0]), type(old_pairs[0].state)
            template = old_pairs[0].state.status
            inactive = _status_like(template, 0)
        else:
            Pair, State, Status = pair_types()
            inactive = Status(0)
        for i in fresh:  # appended in candidate order, as the reference does
            a, b = int(st["ea"][i]), int(st["eb"][i])
            pairs.append(Pair(elem_a=a, elem_b=b, nodes_a=conn[a].copy(), nodes_b=conn[b].copy(),
                              state=State(status=inactive), radius_a=float(r[a]), radius_b=float(r[b]),
                              core_radius_a=float(cr[a]), core_radius_b=float(cr[b])))
        cl = cands.view(-1, 2).cpu().numpy()
        return DetectCandidatesResult(manager=_replace_pairs(manager, pairs),
                                      candidates=[(int(x), int(y)) for x, y in cl], n_pairs=len(pairs))


class GpuUpdateGeometryProcess:
    """``UpdateGeometryProcess`` (``contact/_manager_process.py:312-408``) on the GPU.

    ``process(inp)`` takes an object with the fields of ``UpdateGeometryInput``
    (manager, node_coords, allow_deactivation, freeze_active_set) and returns
    the manager with every pair's s, t, gap and frame updated at node_coords and,
    unless frozen, the active-set hysteresis applied with config.g_on/g_off.
    """

    def __init__(self, device=None) -> None:
        self._device = device

    def process(self, inp) -> UpdateGeometryResult:
        manager = inp.manager
        config = manager.config
        pairs = list(manager.pairs)
        if not pairs:
            return UpdateGeometryResult(manager=manager, n_active=0)
        coords = np.asarray(inp.node_coords, dtype=float).reshape(-1, 3)
        freeze = bool(getattr(inp, "freeze_active_set", False))
        cp = _contact_params(g_on=getattr(config, "g_on", 0.0), g_off=getattr(config, "g_off", 1e-6),
                             allow_deactivation=bool(getattr(inp, "allow_deactivation", True)))
        if getattr(config, "coating_stiffness", 0.0) > 0.0:
            _coated_geometry(pairs, coords, cp, not freeze, self._device)
        else:
            batch = PairBatch(pairs, coords.shape[0], coords=coords, device=self._device)
            batch.narrowphase(cp, not freeze)
            _write_geometry(pairs, batch.state(), range(len(pairs)), not freeze)
        n_active = sum(1 for p in pairs if _code(p.state.status) != 0)
        return UpdateGeometryResult(manager=_replace_pairs(manager, pairs), n_active=n_active)


# ----------------------------------------------------------------------------- beam


def _rotvec_to_rotmat(th: np.ndarray) -> np.ndarray:
    """Rodrigues' formula for a stack of rotation vectors (small angles by series)."""
    th = np.asarray(th, dtype=float).reshape(-1, 3)
    a = np.linalg.norm(th, axis=1)
    K = np.zeros((th.shape[0], 3, 3))
    K[:, 0, 1], K[:, 0, 2], K[:, 1, 2] = -th[:, 2], th[:, 1], -th[:, 0]
    K[:, 1, 0], K[:, 2, 0], K[:, 2, 1] = th[:, 2], -th[:, 1], th[:, 0]
    small = a < 1e-12
    s1 = np.where(small, 1.0 - a**2 / 6.0, np.sin(a) / np.where(small, 1.0, a))
    s2 = np.where(small, 0.5 - a**2 / 24.0, (1.0 - np.cos(a)) / np.where(small, 1.0, a) ** 2)
    return np.eye(3)[None] + s1[:, None, None] * K + s2[:, None, None] * (K @ K)


class GpuCRBeamAssembler:
    """``ULCRBeamAssembler`` (``elements/_beam_assembler.py:19-196``) on the GPU.

    ``assemble_tangent(u_incr)`` and ``assemble_internal_force(u_incr)`` run the
    CR Timoshenko element kernels on the current reference configuration;
    ``update_reference`` moves it by the converged increment; ``checkpoint`` /
    ``rollback`` save and restore it; ``assemble_mass`` is the lumped diagonal
    (``elements/_beam_cr.py:267-296``).  ``precision="mixed"`` selects the float
    element kernel with quaternion frames.
    """

    def __init__(self, node_coords, connectivity, E: float, G: float, A: float, Iy: float, Iz: float, J: float,
                 kappa_y: float, kappa_z: float = 0.0, *, v_ref=None, scf: float | None = None,
                 precision: str = "fp64", device=None):
        coords = np.asarray(node_coords, dtype=float).reshape(-1, 3)
        self.connectivity = np.asarray(connectivity)
        self.n_nodes = coords.shape[0]
        self.ndof = 6 * self.n_nodes
        self.E, self.G, self.A, self.Iy, self.Iz, self.J = E, G, A, Iy, Iz, J
        self.kappa_y = kappa_y
        self.kappa_z = kappa_z if kappa_z > 0 else kappa_y
        self.v_ref = v_ref
        self.scf = scf
        self.mesh = DeviceMesh(coords, self.connectivity, 0.0, device=device)
        sec = {"E": E, "G": G, "A": A, "Iy": Iy, "Iz": Iz, "J": J, "kappa_y": self.kappa_y,
               "kappa_z": self.kappa_z, "scf": scf}
        self.beam = DeviceBeam(self.mesh, sec, v_ref=v_ref)
        self.precision = {"fp64": L.XK_FP64, "mixed": L.XK_MIXED}[precision]
        dev = self.mesh.device
        self._elem32 = torch.zeros(L.ELEM32_STRIDE * max(self.mesh.n_elems, 1), dtype=torch.float32, device=dev)
        self._node32 = torch.zeros(L.NODE32_STRIDE * max(self.n_nodes, 1), dtype=torch.float32, device=dev)
        self._prepare32()
        self.R_ref = np.tile(np.eye(3), (self.n_nodes, 1, 1))
        self._u_total_accum = np.zeros(self.ndof)
        self._ckpt = None

    @property
    def coords_ref(self) -> np.ndarray:
        return self.mesh.X.view(-1, 3).cpu().numpy()

    def _prepare32(self):
        if self.precision == L.XK_MIXED:
            L.call("xk_beam_prepare32", C.byref(self.mesh.c), ptr(self.beam.elem_ref), ptr(self._elem32),
                   stream_handle())

    def _run(self, u_incr, f, K):
        u = _dev_vec(u_incr, self.mesh.device)
        if self.precision == L.XK_FP64:
            self.beam.assemble(u, L.XK_FP64, f, K)
        else:
            L.call("xk_nodes_prepare", C.byref(self.mesh.c), ptr(u), None, ptr(self._node32), stream_handle())
            L.call("xk_beam_assemble32", C.byref(self.mesh.c), C.byref(self.beam.section), ptr(self._elem32),
                   C.byref(self.beam.plan), ptr(self._node32), ptr(f), ptr(K), stream_handle())

    def assemble_tangent(self, u_incr) -> sp.csr_matrix:
        nb = self.beam.nnzb
        K = torch.zeros(36 * max(nb, 1), dtype=self.beam.k_dtype(self.precision), device=self.mesh.device)
        f = torch.zeros(self.ndof, dtype=torch.float64, device=self.mesh.device)
        self._run(u_incr, f, K)
        return self.beam.to_csr(K)

    def assemble_internal_force(self, u_incr) -> np.ndarray:
        f = torch.zeros(self.ndof, dtype=torch.float64, device=self.mesh.device)
        self._run(u_incr, f, None)
        return f.cpu().numpy()

    def update_reference(self, u_incr) -> None:
        u = np.asarray(u_incr, dtype=float).reshape(-1, 6)
        X = self.coords_ref + u[:, :3]
        self.mesh.set_coords(X)
        self.R_ref = self.R_ref @ _rotvec_to_rotmat(u[:, 3:])
        self._u_total_accum = self._u_total_accum + u.ravel()
        self.beam.update_reference_frames()
        self._prepare32()

    def checkpoint(self) -> None:
        self._ckpt = (self.coords_ref.copy(), self.R_ref.copy(), self._u_total_accum.copy())

    def rollback(self) -> None:
        if self._ckpt is not None:
            X, R, acc = self._ckpt
            self.mesh.set_coords(X)
            self.R_ref, self._u_total_accum = R.copy(), acc.copy()
            self.beam.update_reference_frames()
            self._prepare32()

    @property
    def u_total_accum(self) -> np.ndarray:
        return self._u_total_accum

    def get_total_displacement(self, u_incr) -> np.ndarray:
        return self._u_total_accum + np.asarray(u_incr, dtype=float)

    def assemble_mass(self, rho: float, *, lumped: bool = True) -> sp.csr_matrix:
        if not lumped:
            raise NotImplementedError("only the lumped mass matrix is on the GPU path (lumped=True)")
        m = torch.zeros(self.ndof, dtype=torch.float64, device=self.mesh.device)
        self.beam.lumped_mass(rho, m)
        return sp.diags(m.cpu().numpy(), format="csr")
