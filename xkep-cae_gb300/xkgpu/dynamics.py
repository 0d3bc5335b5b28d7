"""Time integration on the device: ``GpuGeneralizedAlpha`` and ``QuasiStatic``.

``GpuGeneralizedAlpha`` is ``GeneralizedAlphaProcess``
(``xkep_cae/time_integration/strategy.py:96-232``) with a lumped mass and no
damping: the same methods (``predict``, ``correct``, ``effective_stiffness``,
``effective_residual``, ``checkpoint`` / ``restore_checkpoint``,
``set_initial_state``, ``is_dynamic``), the state vectors on the device and the
element-wise updates in the xkgpu kernels.  Vectors passed as NumPy arrays are
returned as NumPy arrays; device tensors stay on the device.  The mass term of
the effective stiffness can be added on the host (scipy, as the reference
returns it) or into the engine's block matrix (``add_mass_to``).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib as L
from .device import as_dev, ptr, require_cuda, stream_handle


def alpha_parameters(rho_inf: float):
    """(alpha_m, alpha_f, gamma, beta) of Chung & Hulbert (``strategy.py:133-136``)."""
    am = (2.0 * rho_inf - 1.0) / (rho_inf + 1.0)
    af = rho_inf / (rho_inf + 1.0)
    return am, af, 0.5 - am + af, 0.25 * (1.0 - am + af) ** 2


class QuasiStatic:
    """``QuasiStaticProcess``: no inertia (identity predictor and effective terms)."""

    is_dynamic = False

    def predict(self, u, dt):
        return u

    def correct(self, u, du, dt):
        return None

    def effective_stiffness(self, K, dt):
        return K

    def effective_residual(self, R, dt):
        return R

    def checkpoint(self):
        return None

    def restore_checkpoint(self):
        return None


class GpuGeneralizedAlpha:
    is_dynamic = True

    def __init__(self, mass_matrix, *, damping_matrix=None, rho_inf: float = 0.9, device=None):
        if damping_matrix is not None:
            raise NotImplementedError("the GPU time integrator takes no damping matrix (lumped mass, undamped)")
        self.device = require_cuda(device)
        if sp.issparse(mass_matrix):
            off = mass_matrix - sp.diags(mass_matrix.diagonal())
            if off.nnz and abs(off).max() > 0.0:
                raise ValueError("the GPU time integrator needs a lumped (diagonal) mass matrix")
            m = mass_matrix.diagonal()
        else:
            m = mass_matrix
        self.m = as_dev(m, torch.float64, self.device)
        self.rho_inf = rho_inf
        self.alpha_m, self.alpha_f, self.gamma, self.beta = alpha_parameters(rho_inf)
        n = self.m.numel()
        z = lambda: torch.zeros(n, dtype=torch.float64, device=self.device)  # noqa: E731
        self.vel, self.acc, self._vel_old, self._acc_old, self._u_pred, self._v_pred = z(), z(), z(), z(), z(), z()
        self._ckpt = None

    @property
    def n(self) -> int:
        return self.m.numel()

    def _in(self, x):
        return x if isinstance(x, torch.Tensor) and x.device == self.device else as_dev(x, torch.float64, self.device)

    @staticmethod
    def _out(like, x):
        return x if isinstance(like, torch.Tensor) else x.cpu().numpy()

    def set_initial_state(self, velocity=None, acceleration=None):
        if velocity is not None:
            self.vel.copy_(self._in(velocity))
        if acceleration is not None:
            self.acc.copy_(self._in(acceleration))

    def predict(self, u, dt: float):
        ud = self._in(u)
        L.call("xk_genalpha_predict", self.n, ptr(ud), ptr(self.vel), ptr(self.acc), ptr(self._vel_old),
               ptr(self._acc_old), ptr(self._u_pred), ptr(self._v_pred), float(dt), self.beta, self.gamma,
               stream_handle())
        return self._out(u, self._u_pred.clone())

    def correct(self, u, du, dt: float) -> None:
        ud = self._in(u)
        L.call("xk_genalpha_correct", self.n, ptr(ud), ptr(self._u_pred), ptr(self._v_pred), ptr(self.acc),
               ptr(self.vel), float(dt), self.beta, self.gamma, stream_handle())

    def mass_coefficient(self, dt: float) -> float:
        """(1 - alpha_m) c0, the factor of M in the effective stiffness; 0 for dt ~ 0."""
        if dt < 1e-30:
            return 0.0
        return (1.0 - self.alpha_m) * (1.0 / (self.beta * dt**2))

    def effective_stiffness(self, K, dt: float):
        """K + (1 - alpha_m) c0 M as a scipy matrix (the reference's return type)."""
        if dt < 1e-30:
            return K
        return (K + sp.diags(self.mass_coefficient(dt) * self.m.cpu().numpy())).tocsr()

    def add_mass_to(self, K_vals: torch.Tensor, diag_index: torch.Tensor, dt: float, precision: int):
        """Add (1 - alpha_m) c0 M into a device block matrix at its diagonal value indices."""
        c = self.mass_coefficient(dt)
        if c != 0.0:
            L.call("xk_add_diagonal", self.n, ptr(diag_index), ptr(self.m), c, int(precision), ptr(K_vals),
                   stream_handle())

    def effective_residual(self, R, dt: float):
        Rd = self._in(R)
        out = torch.empty_like(Rd)
        L.call("xk_genalpha_residual", self.n, ptr(Rd), ptr(self.m), ptr(self.acc), ptr(self._acc_old),
               self.alpha_m, ptr(out), stream_handle())
        return self._out(R, out)

    def checkpoint(self):
        self._ckpt = (self.vel.clone(), self.acc.clone())

    def restore_checkpoint(self):
        if self._ckpt is not None:
            self.vel.copy_(self._ckpt[0])
            self.acc.copy_(self._ckpt[1])
