"""Strand workloads with the material, section, penalty and contact settings of the benchmarks.

Steel wires (E = 200 GPa, nu = 0.3) in mm-N-MPa units, circular sections with
Cowper's shear factor (``xkep_cae/elements/_beam_section.py:59-65,129-136``),
penalty ``k_pen = 1e3 * E A / L_mean`` (``AutoEALPenalty``,
``xkep_cae/contact/penalty/strategy.py:111-131``) or, for the solver runs that
take the reference's default, ``k_pen = 0.1 * 12 E I / L_mean^3``
(``AutoBeamEIPenalty``, ``strategy.py:59-101``; the contact config's default
``k_pen_mode = "beam_ei"``, ``k_pen_scale = 0.1``, ``contact/_contact_pair.py:87-88``;
what ``ContactFrictionProcess`` uses when the setup's k_pen is 0,
``contact/solver/process.py:203-211``), mu = 0.1, k_t_ratio = 0.5,
same-layer pairs excluded.  Positions are perturbed by N(0, (1e-3 d)^2) and
rotations by N(0, (1e-3 rad)^2) from ``numpy.random.default_rng(seed)``.
"""

from __future__ import annotations

import math
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import strand as S

E_STEEL = 2.0e5
NU_STEEL = 0.3


def circle_section(d: float, E: float = E_STEEL, nu: float = NU_STEEL) -> dict:
    r = d / 2.0
    kappa = 6.0 * (1.0 + nu) / (7.0 + 6.0 * nu)
    return {"E": E, "G": E / (2.0 * (1.0 + nu)), "A": math.pi * r * r, "Iy": math.pi * d**4 / 64.0,
            "Iz": math.pi * d**4 / 64.0, "J": math.pi * d**4 / 32.0, "kappa_y": kappa, "kappa_z": kappa}


def mean_element_length(coords, conn) -> float:
    conn = np.asarray(conn)
    return float(np.mean(np.linalg.norm(coords[conn[:, 1]] - coords[conn[:, 0]], axis=1)))


@dataclass
class Workload:
    name: str
    strand: S.Strand
    section: dict
    u: np.ndarray
    k_pen: float
    mu: float | np.ndarray = 0.1  # one value, or one per element (batched strands)
    k_t_ratio: float = 0.5
    smoothing_delta: float = 0.0
    meta: dict = field(default_factory=dict)

    def engine_kwargs(self) -> dict:
        return dict(layer=self.strand.elem_layer, k_pen=self.k_pen, k_t_ratio=self.k_t_ratio, mu=self.mu,
                    smoothing_delta=self.smoothing_delta)


def beam_ei_penalty(section: dict, l_mean: float, scale: float = 0.1) -> float:
    """``AutoBeamEIPenalty._compute`` with one contact pair: scale * 12 E I / L^3."""
    return scale * 12.0 * section["E"] * section["Iy"] / l_mean**3


def strand_workload(name: str, n_wires: int, d: float, pitch: float, n_pitches: float, n_el_per_pitch: int, *,
                    gap_frac: float = -0.005, seed: int = 0, mu: float = 0.1, compress_layer: int | None = None,
                    compress_frac: float = 0.0, penalty: str = "ea") -> Workload:
    n_el = int(round(n_el_per_pitch * n_pitches))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        st = S.make_strand(n_wires, d, pitch, n_pitches, n_el, gap=gap_frac * d)
    u = S.perturbation(st, seed, sigma_pos=1e-3 * d, sigma_rot=1e-3)
    if compress_layer is not None:
        u = u + S.radial_compression(st, compress_layer, compress_frac * d)
    sec = circle_section(d)
    l_mean = mean_element_length(st.coords, st.conn)
    if penalty == "ea":
        k_pen = 1e3 * sec["E"] * sec["A"] / l_mean
    elif penalty == "beam_ei":
        k_pen = beam_ei_penalty(sec, l_mean)
    else:
        raise ValueError(f"penalty: 'ea' or 'beam_ei', not {penalty!r}")
    return Workload(name, st, sec, u, k_pen, mu=mu, meta={"n_wires": n_wires, "d": d, "pitch": pitch,
                                                          "n_pitches": n_pitches, "n_el_per_pitch": n_el_per_pitch,
                                                          "gap_frac": gap_frac, "seed": seed,
                                                          "compress_layer": compress_layer,
                                                          "compress_frac": compress_frac, "penalty": penalty})


def wires_for_layers(n_layers: int) -> int:
    return 1 + sum(6 * k for k in range(1, n_layers + 1))


# The benchmark strands (wire count, diameter, pitch, pitches, elements per pitch)
CONFIGS = {
    "strand7": dict(n_wires=7, d=2.0, pitch=40.0, n_pitches=1, n_el_per_pitch=16),
    "strand37": dict(n_wires=37, d=2.0, pitch=40.0, n_pitches=4, n_el_per_pitch=32),
    # the 37-wire load-step strand: nominal lay (a gap of -1e-12 d skips the minimum-gap bump) with the
    # outer layer moved radially inward by 0.005 d
    "strand37c": dict(n_wires=37, d=2.0, pitch=40.0, n_pitches=4, n_el_per_pitch=32, gap_frac=-1e-12,
                      compress_layer=3, compress_frac=0.005),
    "strand91": dict(n_wires=91, d=2.0, pitch=40.0, n_pitches=4, n_el_per_pitch=32),
    "strand397": dict(n_wires=wires_for_layers(11), d=0.5, pitch=20.0, n_pitches=4, n_el_per_pitch=24),
    "strand1027": dict(n_wires=wires_for_layers(18), d=0.5, pitch=20.0, n_pitches=4, n_el_per_pitch=24),
}


def batch_workload(name: str = "batch256", n_strands: int = 256, seed: int = 0, d: float = 2.0,
                   pitch: float = 40.0) -> Workload:
    """Independent strands in one mesh: wire counts drawn from {7, 19, 37}, 1-4 pitches, 8-48
    elements per pitch, seeded perturbations, a friction coefficient per strand in [0.05, 0.3].

    The strands lie side by side without touching; ``mu`` of the workload holds
    one coefficient per element and ``meta['instance']`` the strand of every
    element.  The penalty is the batch's 1e3 EA / L_mean.
    """
    rng = np.random.default_rng(seed)
    strands, us, mus = [], [], []
    for k in range(n_strands):
        nw = int(rng.choice([7, 19, 37]))
        npt = int(rng.integers(1, 5))
        epp = int(rng.integers(8, 49))
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            st = S.make_strand(nw, d, pitch, npt, epp * npt, gap=-0.005 * d, allow_coarse=True)
        strands.append(st)
        us.append(S.perturbation(st, seed * 100003 + k, sigma_pos=1e-3 * d, sigma_rot=1e-3))
        mus.append(float(rng.uniform(0.05, 0.3)))
    merged, inst, node_first = S.merge_strands(strands)
    u = np.concatenate(us)
    sec = circle_section(d)
    k_pen = 1e3 * sec["E"] * sec["A"] / mean_element_length(merged.coords, merged.conn)
    mu_elem = np.asarray(mus)[inst]
    return Workload(name, merged, sec, u, k_pen, mu=mu_elem,
                    meta={"n_strands": n_strands, "d": d, "pitch": pitch, "seed": seed, "instance": inst,
                          "node_first": node_first, "mu_instance": np.asarray(mus),
                          "n_wires": [len(s.wires) for s in strands]})


def config_workload(name: str, seed: int = 0) -> Workload:
    if name.startswith("batch"):
        n = int(name[5:]) if name[5:] else 256
        return batch_workload(name, n_strands=n, seed=seed)
    return strand_workload(name, seed=seed, **CONFIGS[name])
