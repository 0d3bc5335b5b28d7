"""CPU oracle of the Generalized-alpha time integration (test infrastructure only).

Restates ``GeneralizedAlphaProcess`` (``xkep_cae/time_integration/strategy.py:96-232``,
Chung & Hulbert 1993) with a lumped (diagonal) mass and no damping, the form
the strand runs use.
"""

from __future__ import annotations

import numpy as np


def parameters(rho_inf: float):
    """(alpha_m, alpha_f, gamma, beta) from the spectral radius (``strategy.py:133-136``)."""
    am = (2.0 * rho_inf - 1.0) / (rho_inf + 1.0)
    af = rho_inf / (rho_inf + 1.0)
    gamma = 0.5 - am + af
    beta = 0.25 * (1.0 - am + af) ** 2
    return am, af, gamma, beta


class GeneralizedAlpha:
    def __init__(self, m_diag: np.ndarray, rho_inf: float = 0.9):
        self.m = np.asarray(m_diag, dtype=float)
        self.am, self.af, self.gamma, self.beta = parameters(rho_inf)
        n = self.m.size
        self.vel, self.acc = np.zeros(n), np.zeros(n)
        self.vel_old, self.acc_old = np.zeros(n), np.zeros(n)
        self.u_pred, self.v_pred = np.zeros(n), np.zeros(n)

    def predict(self, u, dt):
        """``strategy.py:163-174``."""
        self.acc_old = self.acc.copy()
        self.vel_old = self.vel.copy()
        self.u_pred = u + dt * self.vel + 0.5 * dt**2 * (1.0 - 2.0 * self.beta) * self.acc
        self.v_pred = self.vel + dt * (1.0 - self.gamma) * self.acc
        return self.u_pred.copy()

    def correct(self, u, du, dt):
        """``strategy.py:176-185``."""
        if dt < 1e-30:
            return
        c0 = 1.0 / (self.beta * dt**2)
        self.acc = c0 * (u - self.u_pred)
        self.vel = self.v_pred + dt * self.gamma * self.acc

    def effective_stiffness_diag(self, dt):
        """The term added to K's diagonal: (1 - alpha_m) c0 M (``strategy.py:187-200``)."""
        if dt < 1e-30:
            return np.zeros_like(self.m)
        c0 = 1.0 / (self.beta * dt**2)
        return (1.0 - self.am) * c0 * self.m

    def effective_residual(self, R, dt):
        """R + M a_mid, a_mid = (1 - alpha_m) a + alpha_m a_old (``strategy.py:202-216``)."""
        a_mid = (1.0 - self.am) * self.acc + self.am * self.acc_old
        return R + self.m * a_mid
