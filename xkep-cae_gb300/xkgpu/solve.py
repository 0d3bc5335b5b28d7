"""The Newton step's linear system solved on the device.

``LinearSolveProcess`` (``xkep_cae/contact/solver/_newton_steps.py:338-366``)
solves ``K du = -R`` with the Dirichlet DOFs' rows and columns replaced by the
identity, by a direct sparse factorisation on the host.  ``DeviceLinearSolver``
keeps ``K = K_beam + K_c`` in the engine's block matrices and runs BiCGStab
with a block-Jacobi preconditioner (each node's 6x6 diagonal block) in the
``xk_bicgstab`` kernels: no matrix leaves the device, and the only host
synchronisations are the convergence checks (each check interval of
iterations replays as one CUDA graph).
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .device import ptr, stream_handle


class LinearSolveError(RuntimeError):
    """The iterative solve did not reach its tolerance."""


class DeviceLinearSolver:
    """BiCGStab on ``engine.K_beam + engine.K_c`` with Dirichlet identity rows and columns."""

    def __init__(self, engine, *, rtol: float = 1e-10, max_iter: int = 2000, check_every: int = 10,
                 strict: bool = True):
        self.engine = engine
        self.rtol, self.max_iter, self.check_every, self.strict = float(rtol), int(max_iter), int(check_every), strict
        n = engine.mesh.n_nodes
        dev = engine.device
        self.dinv = torch.zeros(36 * max(n, 1), dtype=torch.float64, device=dev)
        self.work = torch.zeros(8 * 6 * max(n, 1) + 2 * L.SOLVE_REDUCE_BLOCKS + 8, dtype=torch.float64, device=dev)
        self.fixed = torch.zeros(6 * max(n, 1), dtype=torch.uint8, device=dev)
        self.sys = L.System()
        self.iterations = 0
        self.rel_res = 0.0
        self.history: list[tuple[int, float]] = []  # (iterations, relative residual) of every solve

    def set_fixed(self, fixed) -> None:
        f = torch.as_tensor(np.asarray(fixed, dtype=np.uint8) if not torch.is_tensor(fixed) else fixed)
        self.fixed[: f.numel()].copy_(f.to(torch.uint8).reshape(-1))

    def _sync(self, K_beam=None) -> L.System:
        e, s = self.engine, self.sys
        s.n_nodes = e.mesh.n_nodes
        s.precision = e.precision
        s.kb_row_ptr, s.kb_col = ptr(e.beam.row_ptr), ptr(e.beam.col)
        s.kb_vals = ptr(e.K_beam if K_beam is None else K_beam)
        s.kb_blk_row, s.kb_low_ptr, s.kb_low_blk = ptr(e.beam.blk_row), ptr(e.beam.low_ptr), ptr(e.beam.low_blk)
        pat = e.pattern
        if pat.nnzb > 0:  # the stored (row <= column) blocks; the kernels add their mirrors
            s.kc_row_ptr, s.kc_col, s.kc_vals = ptr(pat.row_ptr), ptr(pat.col), ptr(e.K_c)
            s.kc_blk_row, s.kc_low_ptr, s.kc_low_blk = ptr(pat.blk_row), ptr(pat.low_ptr), ptr(pat.low_blk)
        else:
            s.kc_row_ptr = s.kc_col = s.kc_vals = s.kc_blk_row = s.kc_low_ptr = s.kc_low_blk = None
        s.fixed = ptr(self.fixed)
        return s

    def matvec(self, x: torch.Tensor, y: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """y = A x (A the Dirichlet-masked K_beam + K_c)."""
        y = torch.empty_like(x) if y is None else y
        L.call("xk_system_spmv", C.byref(self._sync()), ptr(x), ptr(y), stream_handle(stream))
        return y

    def solve(self, b: torch.Tensor, x0: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """x with ``A x = b`` from ``x0`` (zero by default); b, x double on the device."""
        b = b.to(torch.float64).contiguous()
        x = torch.zeros_like(b) if x0 is None else x0.to(torch.float64).clone()
        sysc = self._sync()
        h = stream_handle(stream)
        L.call("xk_system_block_jacobi", C.byref(sysc), ptr(self.dinv), h)
        it, rr = C.c_int32(0), C.c_double(0.0)
        L.call("xk_bicgstab", C.byref(sysc), ptr(b), ptr(x), ptr(self.dinv), ptr(self.work), self.max_iter,
               self.check_every, self.rtol, C.byref(it), C.byref(rr), h)
        self.iterations, self.rel_res = int(it.value), float(rr.value)
        self.history.append((self.iterations, self.rel_res))
        if self.strict and not (self.rel_res <= self.rtol):
            raise LinearSolveError(f"BiCGStab: relative residual {self.rel_res:.3e} after {self.iterations} "
                                   f"iterations (tolerance {self.rtol:.1e})")
        return x
