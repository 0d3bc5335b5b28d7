"""The oracle as an assembly backend of ``xkgpu.solver.ContactFrictionSolver`` (test infrastructure).

``OracleBackend`` runs detection, the frozen-geometry contact iteration and
the beam assembly with ``oracle/`` on the host, in the call order of the
reference's ``ContactForceAssemblyProcess`` / ``TangentAssemblyProcess``
(``xkep_cae/contact/solver/_newton_steps.py:79-135,289-313``); ``TorchGA``
puts the oracle's Generalized-alpha integrator behind the solver's torch
interface.  With these the solver loop runs entirely on the CPU, which pins
the loop itself against the reference's own solver run.
"""

from __future__ import annotations

import numpy as np
import torch

from oracle import beam as ob
from oracle import contact as oc
from oracle import dynamics as od


class OracleBackend:
    def __init__(self, X, conn, radii, section: dict, *, layer, k_pen, k_t_ratio, mu, smoothing_delta=0.0):
        self.X = np.asarray(X, dtype=float)
        self.conn = np.asarray(conn)
        self.radii = np.broadcast_to(np.asarray(radii, dtype=float), (len(self.conn),)).copy()
        self.layer = np.asarray(layer)
        self.sec = ob.Section(**section, scf=None)
        self.k_pen, self.k_t_ratio, self.mu, self.sd = k_pen, k_t_ratio, mu, smoothing_delta
        self.ndof = 6 * len(self.X)
        self.device = torch.device("cpu")
        self.table = oc.empty_table()
        self.K = None
        self.detections = []

    def detect(self, u: torch.Tensor) -> dict:
        x = oc.deformed_coords(self.X, u.numpy())
        self.table, cands, raw = oc.detect(self.table, x, self.conn, self.radii, elem_layer=self.layer,
                                           exclude_same_layer=True)
        self.table = oc.update_geometry(self.table, x)
        self.detections.append(len(cands))
        return {"candidates": len(cands), "pairs": len(self.table["ea"])}

    def assemble(self, u, u_ref, f_ext, fixed_u8):
        un = u.numpy()
        self.table, fc, Kc, _ = oc.contact_iteration(self.table, self.X, un, u_ref.numpy(), self.ndof,
                                                     k_pen=self.k_pen, k_t_ratio=self.k_t_ratio, mu_eff=self.mu,
                                                     smoothing_delta=self.sd)
        Kb, fb = ob.assemble_beam(self.X, self.conn, un, self.sec)
        self.K = (Kb + Kc).tocsr()
        R = fb + fc - f_ext.numpy()
        R[fixed_u8.numpy().astype(bool)] = 0.0
        return torch.as_tensor(R), torch.as_tensor(fc)

    def internal_force(self, u):
        _, f = ob.assemble_beam(self.X, self.conn, u.numpy(), self.sec, stiffness=False)
        return torch.as_tensor(f)

    def n_active(self) -> int:
        return int((self.table["p_n"] > 0.0).sum())

    def K_csr(self):
        return self.K


class TorchGA:
    """``oracle.dynamics.GeneralizedAlpha`` with the checkpoints and torch vectors the solver uses."""

    is_dynamic = True

    def __init__(self, m_diag, rho_inf: float = 0.9):
        self.ga = od.GeneralizedAlpha(m_diag, rho_inf)
        self.m = torch.as_tensor(np.asarray(m_diag, dtype=float))
        self._ckpt = None

    def predict(self, u, dt):
        return torch.as_tensor(self.ga.predict(u.numpy(), dt))

    def correct(self, u, du, dt):
        self.ga.correct(u.numpy(), None, dt)

    def effective_residual(self, R, dt):
        return torch.as_tensor(self.ga.effective_residual(R.numpy(), dt))

    def mass_coefficient(self, dt):
        if dt < 1e-30:
            return 0.0
        return (1.0 - self.ga.am) * (1.0 / (self.ga.beta * dt**2))

    def checkpoint(self):
        self._ckpt = (self.ga.vel.copy(), self.ga.acc.copy())

    def restore_checkpoint(self):
        if self._ckpt is not None:
            self.ga.vel, self.ga.acc = self._ckpt[0].copy(), self._ckpt[1].copy()
