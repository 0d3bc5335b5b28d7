"""Twisted-wire strand meshes and seeded states: the synthetic workloads.

This is the input generator for the assembly path, not part of it.  It builds
the same layered helical strand as xkep-cae's mesh generator
(``xkep_cae/mesh/_twisted_wire.py:150-383``): wire 0 is a straight core, layer
``k`` holds ``6k`` wires on a helix of lay radius ``k*(d_eff+gap)``, odd layers
twist one way and even layers the other, every wire is a chain of ``n_el``
two-node elements, and a non-negative ``gap`` is raised to the chord-sagitta
"minimum safe gap" (``_twisted_wire.py:127-147,307-326``).  Node coordinates
follow the reference's own arithmetic (``i*L/(n-1)`` for helices, ``linspace``
for the core) so that a mesh made here equals the reference mesh bit for bit on
the same platform.

Units are mm-N-MPa throughout.
"""

from __future__ import annotations

import math
import warnings
from dataclasses import dataclass, field

import numpy as np


@dataclass(frozen=True)
class WireInfo:
    """Placement of one wire in the strand cross-section."""

    wire_id: int
    layer: int
    angle_offset: float
    lay_radius: float
    lay_direction: int


@dataclass
class Strand:
    """A strand mesh: nodes, two-node elements and per-element attributes."""

    coords: np.ndarray  # (n_nodes, 3) float64
    conn: np.ndarray  # (n_elems, 2) int32
    elem_layer: np.ndarray  # (n_elems,) int32 layer index of each element's wire
    radii: np.ndarray  # (n_elems,) float64 wire radius per element
    wires: tuple[WireInfo, ...]
    wire_diameter: float
    pitch: float
    length: float
    n_elems_per_wire: int
    node_offset: int = 0  # first node id when several strands share one mesh
    meta: dict = field(default_factory=dict)

    @property
    def n_nodes(self) -> int:
        return int(self.coords.shape[0])

    @property
    def n_elems(self) -> int:
        return int(self.conn.shape[0])

    @property
    def ndof(self) -> int:
        return 6 * self.n_nodes

    def layer_map(self) -> dict[int, int]:
        """``{element: layer}`` as the reference's ``elem_layer_map`` expects."""
        return {int(e): int(l) for e, l in enumerate(self.elem_layer)}


def layer_counts(n_wires: int) -> list[int]:
    """Wires per layer: ``[1, 6, 12, ...]`` with a partial last layer."""
    if n_wires == 3:
        return [0, 3]
    counts = [1]
    remaining = n_wires - 1
    k = 1
    while remaining > 0:
        take = min(6 * k, remaining)
        counts.append(take)
        remaining -= take
        k += 1
    return counts


def min_safe_gap(n_wires: int, wire_radius: float, n_elems_per_pitch: float) -> float:
    """Chord-sagitta gap that keeps polygonal helices of adjacent layers apart.

    Two times the sagitta of a chord spanning ``2*pi/n_per_pitch`` on a circle of
    radius ``d``, times a safety factor of two.
    """
    if n_wires <= 1 or n_elems_per_pitch < 1:
        return 0.0
    d_eff = 2.0 * wire_radius
    sagitta = d_eff * (1.0 - math.cos(math.pi / n_elems_per_pitch))
    return 2.0 * sagitta * 2.0


def wire_layout(n_wires: int, wire_radius: float, gap: float, lay_direction: int = 1) -> list[WireInfo]:
    """Cross-section placement of every wire (core first, then layer by layer)."""
    d_eff = 2.0 * wire_radius
    wires: list[WireInfo] = []
    if n_wires == 3:
        r = (d_eff + gap) / math.sqrt(3.0)
        return [WireInfo(k, 1, 2.0 * math.pi * k / 3.0, r, lay_direction) for k in range(3)]
    wires.append(WireInfo(0, 0, 0.0, 0.0, 0))
    remaining = n_wires - 1
    k = 1
    while remaining > 0:
        slots = 6 * k
        take = min(slots, remaining)
        r = k * (d_eff + gap)
        direction = lay_direction if k % 2 == 1 else -lay_direction
        for j in range(take):
            wires.append(WireInfo(len(wires), k, 2.0 * math.pi * j / slots, r, direction))
        remaining -= take
        k += 1
    return wires


def make_strand(
    n_wires: int,
    wire_diameter: float,
    pitch: float,
    n_pitches: float,
    n_elems_per_wire: int,
    *,
    gap: float = 0.0,
    lay_direction: int = 1,
    min_elems_per_pitch: int = 16,
    allow_coarse: bool = False,
) -> Strand:
    """Build a layered helical strand.

    ``allow_coarse`` admits fewer than 16 elements per pitch, which the
    reference generator rejects (``_twisted_wire.py:291-305``); the batched
    many-strand workload needs 8-15 elements per pitch.
    """
    r_w = wire_diameter / 2.0
    length = n_pitches * pitch
    per_pitch = n_elems_per_wire * pitch / length if length > 0 else float(n_elems_per_wire)
    if n_wires > 1 and not allow_coarse and per_pitch < min_elems_per_pitch:
        raise ValueError(
            f"{per_pitch:.1f} elements per pitch is below the minimum of {min_elems_per_pitch}"
        )
    if n_wires > 1 and gap >= 0:
        g_min = min_safe_gap(n_wires, r_w, per_pitch)
        if gap < g_min:
            warnings.warn(f"gap {gap:.6f} raised to the minimum safe gap {g_min:.6f}", stacklevel=2)
            gap = g_min
    wires = wire_layout(n_wires, r_w, gap, lay_direction)

    npw = n_elems_per_wire + 1
    coords = np.zeros((n_wires * npw, 3))
    conn = np.zeros((n_wires * n_elems_per_wire, 2), dtype=np.int32)
    elem_layer = np.zeros(n_wires * n_elems_per_wire, dtype=np.int32)
    idx = np.arange(npw)
    # core wire: numpy linspace arithmetic (i * step, last point pinned)
    core_z = np.linspace(0.0, length, npw)
    # helices: (i * L) / (n - 1) in double, as a Python float expression
    helix_z = np.array([i * length / (npw - 1) for i in range(npw)])
    for w in wires:
        n0 = w.wire_id * npw
        if w.lay_radius < 1e-15:
            coords[n0 : n0 + npw, 2] = core_z
        else:
            for i in range(npw):
                z = helix_z[i]
                th = w.lay_direction * 2.0 * math.pi * z / pitch + w.angle_offset
                coords[n0 + i, 0] = w.lay_radius * math.cos(th)
                coords[n0 + i, 1] = w.lay_radius * math.sin(th)
                coords[n0 + i, 2] = z
        e0 = w.wire_id * n_elems_per_wire
        conn[e0 : e0 + n_elems_per_wire, 0] = n0 + idx[:-1]
        conn[e0 : e0 + n_elems_per_wire, 1] = n0 + idx[1:]
        elem_layer[e0 : e0 + n_elems_per_wire] = w.layer
    return Strand(
        coords=coords,
        conn=conn,
        elem_layer=elem_layer,
        radii=np.full(conn.shape[0], r_w),
        wires=tuple(wires),
        wire_diameter=wire_diameter,
        pitch=pitch,
        length=length,
        n_elems_per_wire=n_elems_per_wire,
        meta={"gap": gap, "n_wires": n_wires, "n_pitches": n_pitches},
    )


def perturbation(strand: Strand, seed: int, *, sigma_pos: float, sigma_rot: float) -> np.ndarray:
    """Seeded Gaussian nodal displacement ``u`` (node-major ``[ux,uy,uz,rx,ry,rz]``)."""
    rng = np.random.default_rng(seed)
    u = np.zeros(strand.ndof)
    uu = u.reshape(-1, 6)
    uu[:, 0:3] = rng.normal(0.0, sigma_pos, (strand.n_nodes, 3))
    uu[:, 3:6] = rng.normal(0.0, sigma_rot, (strand.n_nodes, 3))
    return u


def radial_compression(strand: Strand, layer: int, amount: float) -> np.ndarray:
    """Displacement moving every node of ``layer`` radially inward by ``amount``."""
    u = np.zeros(strand.ndof)
    uu = u.reshape(-1, 6)
    npw = strand.n_elems_per_wire + 1
    for w in strand.wires:
        if w.layer != layer:
            continue
        sl = slice(w.wire_id * npw, (w.wire_id + 1) * npw)
        xy = strand.coords[sl, 0:2]
        r = np.linalg.norm(xy, axis=1, keepdims=True)
        uu[sl, 0:2] = -amount * xy / np.maximum(r, 1e-30)
    return u


def strand_offsets(strands: list[Strand], spacing: float | None = None) -> list[float]:
    """x shift of every strand laid side by side: half-widths (outer lay radius + d) plus a spacing."""
    xs, out = 0.0, []
    for s in strands:
        half = max((w.lay_radius for w in s.wires), default=0.0) + s.wire_diameter
        gap = spacing if spacing is not None else 4.0 * s.wire_diameter
        out.append(xs + half)
        xs += 2.0 * half + gap
    return out


def merge_strands(strands: list[Strand], spacing: float | None = None) -> tuple[Strand, np.ndarray, np.ndarray]:
    """Lay several strands side by side in one mesh (the batched workload).

    Returns the merged strand, the per-element instance id and the first node of
    every instance.  Strands are shifted along x so that no two instances touch.
    """
    offsets = strand_offsets(strands, spacing)
    coords, conns, layers, radii, node_first, inst = [], [], [], [], [], []
    n_off = 0
    for k, s in enumerate(strands):
        c = s.coords.copy()
        c[:, 0] += offsets[k]
        coords.append(c)
        conns.append(s.conn + n_off)
        layers.append(s.elem_layer)
        radii.append(s.radii)
        node_first.append(n_off)
        inst.append(np.full(s.n_elems, k, dtype=np.int32))
        n_off += s.n_nodes
    merged = Strand(
        coords=np.concatenate(coords),
        conn=np.concatenate(conns).astype(np.int32),
        elem_layer=np.concatenate(layers).astype(np.int32),
        radii=np.concatenate(radii),
        wires=(),
        wire_diameter=max(s.wire_diameter for s in strands),
        pitch=0.0,
        length=max(s.length for s in strands),
        n_elems_per_wire=0,
        meta={"instances": len(strands)},
    )
    return merged, np.concatenate(inst), np.asarray(node_first, dtype=np.int64)


def strand_spec(strand: Strand, *, x_offset: float = 0.0, node_first: int = 0, elem_first: int = 0):
    """The device generator's description (``xk_strand_spec``) of a strand built by ``make_strand``."""
    from . import _lib as L

    lay = next((w.lay_direction for w in strand.wires if w.layer == 1), 1)
    return L.StrandSpec(len(strand.wires), strand.n_elems_per_wire, int(lay), 0, strand.wire_diameter,
                        strand.pitch, strand.length, float(strand.meta.get("gap", 0.0)), float(x_offset),
                        int(node_first), int(elem_first))


def generate_on_device(specs: list, device=None):
    """Nodes, connectivity, element layers and radii of the strands ``specs`` (``xk_strand_spec``) on the GPU.

    The specs must tile the mesh in order (``node_first`` / ``elem_first``
    ascending, each strand right after the previous one).  Returns
    ``(X (n_nodes, 3) float64, conn (n_elems, 2) int32, layer int32, radii float64)`` device tensors.
    """
    import ctypes as C

    import torch

    from . import _lib as L
    from .device import ptr, require_cuda, stream_handle

    dev = require_cuda(device)
    n_nodes = sum(s.n_wires * (s.n_elems_per_wire + 1) for s in specs)
    n_elems = sum(s.n_wires * s.n_elems_per_wire for s in specs)
    raw = (L.StrandSpec * len(specs))(*specs)
    buf = torch.frombuffer(bytearray(bytes(raw)), dtype=torch.uint8).to(dev)
    X = torch.empty(3 * max(n_nodes, 1), dtype=torch.float64, device=dev)
    conn = torch.empty(2 * max(n_elems, 1), dtype=torch.int32, device=dev)
    layer = torch.empty(max(n_elems, 1), dtype=torch.int32, device=dev)
    radii = torch.empty(max(n_elems, 1), dtype=torch.float64, device=dev)
    L.call("xk_strand_generate", ptr(buf), len(specs), n_nodes, n_elems, ptr(X), ptr(conn), ptr(layer), ptr(radii),
           stream_handle(None))
    return X[: 3 * n_nodes].view(-1, 3), conn[: 2 * n_elems].view(-1, 2), layer[:n_elems], radii[:n_elems]
