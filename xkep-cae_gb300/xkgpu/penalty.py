"""Penalty stiffness strategies (``PenaltyStrategy.compute_k_pen(step, total_steps)``).

Scalar host formulas with the reference's class names and constructor
arguments (``contact/penalty/strategy.py:34-266``); the chosen k_pen goes into
the contact parameters of the GPU kernels.
"""

from __future__ import annotations

import math
from dataclasses import dataclass


class ConstantPenalty:
    """k_pen fixed for every step (``penalty/strategy.py:34-55``)."""

    def __init__(self, k_pen: float = 1.0) -> None:
        self._k_pen = k_pen

    def compute_k_pen(self, step: int, total_steps: int) -> float:
        return self._k_pen


class AutoBeamEIPenalty:
    """k_pen = scale * 12 E I / L^3 / max(1, f(n_pairs)), f linear or sqrt (``penalty/strategy.py:58-107``)."""

    def __init__(self, beam_E: float, beam_I: float, L_elem: float, *, n_contact_pairs: int = 1,
                 scale: float = 0.1, scaling: str = "linear") -> None:
        if L_elem <= 0.0:
            raise ValueError(f"L_elem must be positive: {L_elem}")
        k_bend = 12.0 * beam_E * beam_I / L_elem**3
        n = max(1, n_contact_pairs)
        div = max(1.0, math.sqrt(n)) if scaling == "sqrt" else max(1.0, float(n))
        self._k_pen = scale * k_bend / div

    def compute_k_pen(self, step: int, total_steps: int) -> float:
        return self._k_pen


class AutoEALPenalty:
    """k_pen = scale * E A / L (``penalty/strategy.py:110-131``)."""

    def __init__(self, beam_E: float, beam_A: float, L_elem: float, *, scale: float = 1.0) -> None:
        if L_elem <= 0.0:
            raise ValueError(f"L_elem must be positive: {L_elem}")
        self._k_pen = scale * beam_E * beam_A / L_elem

    def compute_k_pen(self, step: int, total_steps: int) -> float:
        return self._k_pen


class ContinuationPenalty:
    """k_pen ramped to the target over ``ramp_steps`` steps (``penalty/strategy.py:134-180``).

    geometric: target * start * ratio**step with ratio = (1/start)**(1/ramp_steps), capped at the target;
    linear: target * (start + (1 - start) * step / ramp_steps).
    """

    def __init__(self, k_pen_target: float, *, start_fraction: float = 0.01, ramp_steps: int = 5,
                 mode: str = "geometric") -> None:
        self._target = k_pen_target
        self._start = max(start_fraction, 1e-30)
        self._ramp = max(1, ramp_steps)
        self._mode = mode

    def compute_k_pen(self, step: int, total_steps: int) -> float:
        if step >= self._ramp:
            return self._target
        if self._mode == "geometric":
            ratio = (1.0 / self._start) ** (1.0 / self._ramp)
            return min(self._target * self._start * ratio**step, self._target)
        return self._target * (self._start + (1.0 - self._start) * step / self._ramp)


@dataclass(frozen=True)
class DynamicPenaltyEstimate:
    k_pen: float
    c0: float
    m_ii: float
    c0_m_ii: float


def dynamic_penalty_estimate(rho_inf: float, dt: float, rho: float, A: float, L_elem: float,
                             scale: float = 0.5) -> DynamicPenaltyEstimate:
    """k_pen = scale * c0 * m_ii with c0 = 1/(beta dt^2), m_ii = rho A L / 2 (``penalty/strategy.py:183-266``)."""
    alpha_m = (2.0 * rho_inf - 1.0) / (rho_inf + 1.0)
    alpha_f = rho_inf / (rho_inf + 1.0)
    beta = 0.25 * (1.0 - alpha_m + alpha_f) ** 2
    c0 = 1.0 / (beta * dt * dt)
    m_ii = rho * A * L_elem / 2.0
    return DynamicPenaltyEstimate(k_pen=scale * c0 * m_ii, c0=c0, m_ii=m_ii, c0_m_ii=c0 * m_ii)
