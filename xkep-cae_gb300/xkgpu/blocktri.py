"""Direct solve of the Newton system on the device, for strand meshes.

``LinearSolveProcess`` (``xkep_cae/contact/solver/_newton_steps.py:338-366``)
factorises ``K`` (Dirichlet rows and columns replaced by the identity) with a
sparse direct solver on the host.  The contact tangents of the strand states
are indefinite, which the device's iterative solve cannot handle
(``xkgpu.solve``), and the host's sparse LU fills badly on them (49 s for one
37-wire system).  A strand, though, is long and thin: numbering the nodes
along its axis, every element and every contact couples nodes a few
cross-sections apart.  ``BlockTridiagonalSolver`` therefore

1. orders the nodes along the axis of the mesh's largest extent (once per
   mesh) and takes the block size ``bn`` (nodes) as the largest distance in
   that order between two nodes of one stored block of K_beam or K_c (per
   contact pattern), so that ``K`` is block tridiagonal;
2. scatters ``K_beam + K_c`` (+ the time integrator's mass term) from the
   engine's block matrices into dense diagonal and off-diagonal blocks
   (``xk_system_blocktri``);
3. factorises with block LU, each diagonal block by an LU with partial
   pivoting on the device (cuSOLVER through ``torch.linalg``), and solves.

All in FP64 on the device; the work is ``nb`` dense factorisations of size
``6 bn`` (37-wire strand: 660, 91-wire strand: about 1,600).
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .device import ptr, stream_handle
from .solve import DeviceLinearSolver


def blocktri_solve(D: torch.Tensor, Lo: torch.Tensor, Up: torch.Tensor, rhs: torch.Tensor) -> torch.Tensor:
    """Solve the block-tridiagonal system (diagonal blocks D, blocks left Lo, right Up; (nb, b, b) each) for
    ``rhs`` (nb, b, k) by block LU without pivoting between blocks and LU with partial pivoting inside the
    diagonal blocks: S_0 = D_0, S_i = D_i - Lo_i S_{i-1}^-1 Up_{i-1}.  D and Up are overwritten (by the
    factors of S_i and by S_i^-1 Up_i).  A singular S_i gives non-finite values, as a singular sparse LU does."""
    nb = D.shape[0]
    pivs = []
    for i in range(nb):
        if i > 0:
            D[i].sub_(Lo[i] @ Up[i - 1])
        lu, piv, _ = torch.linalg.lu_factor_ex(D[i])
        D[i].copy_(lu)
        pivs.append(piv)
        if i < nb - 1:
            Up[i].copy_(torch.linalg.lu_solve(lu, piv, Up[i]))
    y = torch.empty_like(rhs)
    for i in range(nb):
        r = rhs[i] if i == 0 else rhs[i] - Lo[i] @ y[i - 1]
        y[i] = torch.linalg.lu_solve(D[i], pivs[i], r)
    for i in range(nb - 2, -1, -1):
        y[i] -= Up[i] @ y[i + 1]
    return y


class BlockTridiagonalSolver:
    """``K du = -R`` by block LU of the axially ordered system; a ``linear_solve`` for ``ContactFrictionSolver``."""

    def __init__(self, engine, axis: int | None = None):
        self.eng = engine
        dev = engine.device
        X = engine.mesh.X_host if hasattr(engine.mesh, "X_host") else None
        if X is None:
            X = engine.mesh.X.reshape(-1, 3).cpu().numpy()
        X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
        if axis is None:
            axis = int(np.argmax(X.max(0) - X.min(0))) if len(X) else 2
        order = np.lexsort((np.arange(len(X)), X[:, axis]))  # along the axis, ties by node id
        pos = np.empty(len(X), dtype=np.int32)
        pos[order] = np.arange(len(X), dtype=np.int32)
        self.pos = torch.as_tensor(pos, device=dev)
        self.order = torch.as_tensor(order.astype(np.int64), device=dev)
        self.n = len(X)
        self._sysw = DeviceLinearSolver(engine)  # the xk_system view of the engine's matrices
        self.overflow = torch.zeros(1, dtype=torch.int32, device=dev)
        self.bn = 0
        self.nb = 0
        self._buf = None
        self._pattern_version = None
        self.stats = {"solves": 0, "failed": 0}

    def _bandwidth(self) -> int:
        e = self.eng
        pos = self.pos.to(torch.int64)
        bw = 0
        nbb = e.beam.nnzb
        if nbb > 0:
            r = e.beam.blk_row[:nbb].to(torch.int64)
            c = e.beam.col[:nbb].to(torch.int64)
            bw = int((pos[r] - pos[c]).abs().max())
        pat = e.pattern
        if pat.nnzb > 0:
            r = pat.blk_row[: pat.nnzb].to(torch.int64)
            c = pat.col[: pat.nnzb].to(torch.int64)
            bw = max(bw, int((pos[r] - pos[c]).abs().max()))
        return max(bw, 1)

    def _prepare(self):
        ver = getattr(self.eng.pattern, "version", None)
        if self._buf is not None and ver == self._pattern_version:
            return
        bn = min(self._bandwidth(), max(self.n, 1))
        nb = -(-self.n // bn)
        b = 6 * bn
        if self._buf is None or self._buf[0].shape != (nb, b, b):
            self._buf = None
            torch.cuda.empty_cache()
            dev = self.eng.device
            self._buf = tuple(torch.empty((nb, b, b), dtype=torch.float64, device=dev) for _ in range(3))
        self.bn, self.nb = bn, nb
        self._pattern_version = ver

    def __call__(self, backend, R: torch.Tensor, fixed: np.ndarray, mass_diag: torch.Tensor | None):
        self._sysw.set_fixed(fixed)
        self._prepare()
        D, Lo, Up = self._buf
        nb, bn, b = self.nb, self.bn, 6 * self.bn
        sysc = self._sysw._sync()
        L.call("xk_system_blocktri", C.byref(sysc), ptr(self.pos), bn, nb,
               ptr(mass_diag) if mass_diag is not None else None, 1.0, ptr(D), ptr(Lo), ptr(Up), ptr(self.overflow),
               stream_handle(None))
        if int(self.overflow.item()):
            raise RuntimeError("block-tridiagonal solve: a coupling reaches beyond the neighbouring block")
        pad = nb * bn - self.n
        if pad:  # positions past the last node: identity rows
            idx = torch.arange(6 * (bn - pad), b, device=D.device)
            D[nb - 1, idx, idx] = 1.0
        # right-hand side -R in the axial order, padded
        rhs = torch.zeros(nb * b, dtype=torch.float64, device=D.device)
        perm = (6 * self.pos.to(torch.int64)[:, None] + torch.arange(6, device=D.device)).reshape(-1)
        rhs[perm] = -R.to(torch.float64)
        y = blocktri_solve(D, Lo, Up, rhs.view(nb, b, 1))
        du = y.reshape(-1)[perm].clone()
        self.stats["solves"] += 1
        if not bool(torch.isfinite(du).all()):
            self.stats["failed"] += 1
        return du
