"""Host logic of the Strategy layer (no GPU): pair packing, status mapping, friction
law helpers, penalty formulas, and method-signature parity with the reference's
Strategy Protocols."""

from __future__ import annotations

import inspect
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import golden

torch = pytest.importorskip("torch")

from oracle import contact as oc  # noqa: E402
from xkgpu import dynamics as D  # noqa: E402
from xkgpu import penalty as P  # noqa: E402
from xkgpu import strategies as S  # noqa: E402


def _pairs(n=5, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        st = S.ContactState(s=rng.random(), t=rng.random(), gap=rng.normal(), normal=rng.normal(size=3),
                            tangent1=rng.normal(size=3), tangent2=rng.normal(size=3), p_n=abs(rng.normal()),
                            z_t=rng.normal(size=2), k_pen=1.0 + i, k_t=0.5 + i, q_trial_norm=rng.random(),
                            status=S.ContactStatus(i % 3), stick=bool(i % 2), dissipation=rng.random())
        out.append(S.ContactPair(elem_a=2 * i, elem_b=2 * i + 7, nodes_a=np.array([3 * i, 3 * i + 1]),
                                 nodes_b=np.array([3 * i + 40, 3 * i + 41]), state=st, radius_a=0.1 * (i + 1),
                                 radius_b=0.2))
    return out


def test_pack_pairs_layout():
    ps = _pairs()
    d = S.pack_pairs(ps)
    assert d["nodes"].shape == (5, 4) and d["normal"].shape == (5, 3) and d["z_t"].shape == (5, 2)
    for i, p in enumerate(ps):
        assert list(d["nodes"][i]) == [*p.nodes_a, *p.nodes_b]
        assert d["status"][i] == p.state.status.value
        assert np.array_equal(d["t1"][i], p.state.tangent1)
        assert d["ra"][i] == p.radius_a and d["k_t"][i] == p.state.k_t
    empty = S.pack_pairs([])
    assert empty["nodes"].shape == (0, 4) and empty["normal"].shape == (0, 3)


def test_status_follows_caller_type():
    assert S._status_like(S.ContactStatus.ACTIVE, 2) is S.ContactStatus.SLIDING
    assert S._status_like(1, 0) == 0 and isinstance(S._status_like(1, 0), int)
    p = S._evolve(_pairs(1)[0], p_n=3.5)
    assert p.state.p_n == 3.5 and isinstance(p.state, S.ContactState)


def test_mu_ramp_and_friction_tangent():
    assert S.mu_effective(0.3, 5, 0) == 0.3
    assert S.mu_effective(0.3, 1, 4) == pytest.approx(0.075)
    assert S.mu_effective(0.3, 9, 4) == 0.3
    assert np.array_equal(S.friction_tangent_2x2(2.0, 1.0, 0.1, np.array([0.3, 0.4]), 0.9, True), 2.0 * np.eye(2))
    # slip: against the oracle's consistent tangent
    t = oc.new_pairs(np.array([[0, 1]]), np.array([[0, 1], [2, 3]]), np.array([0.1, 0.1]))
    t["p_n"][:] = 2.0
    t["k_pen"][:] = 10.0
    t["k_t"][:] = 5.0
    t["t1"][:] = [1.0, 0.0, 0.0]
    t["t2"][:] = [0.0, 1.0, 0.0]
    t["nodes"] = np.array([[0, 1, 2, 3]])
    u = np.zeros(24)
    u[6 * 2 + 0] = 0.3
    u[6 * 3 + 1] = 0.2
    t2, _, _, fr = oc.friction_evaluate(t, u, None, 24, 10.0, 0.5, 0.1)
    assert not t2["stick"][0]
    D = S.friction_tangent_2x2(t2["k_t"][0], t2["p_n"][0], 0.1, t2["z_t"][0], t2["q_trial_norm"][0], False)
    assert np.allclose(D, fr["D"][0], rtol=1e-14, atol=0)


def test_penalty_strategies():
    z = golden("strand7")
    X, conn = z["X"], z["conn"]
    L_mean = float(np.mean(np.linalg.norm(X[conn[:, 1]] - X[conn[:, 0]], axis=1)))
    # the fixtures' k_pen came from the reference's AutoEALPenalty(scale=1e3)
    assert P.AutoEALPenalty(float(z["E"]), float(z["A"]), L_mean, scale=1e3).compute_k_pen(0, 1) == float(z["k_pen"])
    e = P.AutoBeamEIPenalty(2e5, 0.785, 1.5, n_contact_pairs=16, scale=0.1, scaling="sqrt")
    assert e.compute_k_pen(3, 10) == pytest.approx(0.1 * 12 * 2e5 * 0.785 / 1.5**3 / 4.0)
    with pytest.raises(ValueError):
        P.AutoEALPenalty(1.0, 1.0, 0.0)
    c = P.ContinuationPenalty(1e4, start_fraction=0.01, ramp_steps=4)
    assert c.compute_k_pen(0, 10) == pytest.approx(100.0)
    assert c.compute_k_pen(2, 10) == pytest.approx(1e3)
    assert c.compute_k_pen(4, 10) == 1e4
    lin = P.ContinuationPenalty(1e4, start_fraction=0.2, ramp_steps=4, mode="linear")
    assert lin.compute_k_pen(2, 10) == pytest.approx(1e4 * 0.6)
    assert P.ConstantPenalty(7.0).compute_k_pen(1, 2) == 7.0
    d = P.dynamic_penalty_estimate(0.9, 1e-4, 7.85e-9, 0.196, 0.5)
    beta = 0.25 * (1.0 - (0.8 / 1.9) + 0.9 / 1.9) ** 2
    assert d.c0 == pytest.approx(1.0 / (beta * 1e-8))
    assert d.k_pen == pytest.approx(0.5 * d.c0 * 7.85e-9 * 0.196 * 0.25)


def test_rotvec_to_rotmat_matches_oracle():
    from oracle import beam as ob

    rng = np.random.default_rng(3)
    th = np.concatenate([rng.normal(size=(20, 3)), 1e-14 * rng.normal(size=(3, 3)), np.zeros((1, 3))])
    assert np.allclose(S._rotvec_to_rotmat(th), ob.rotvec_to_rotmat(th), rtol=0, atol=1e-14)


def test_gpu_classes_need_a_gpu():
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        S.PairBatch(_pairs(2), 100)


def _reference_protocols() -> dict:
    """Protocol method and parameter names recorded from the reference by ``tests/golden/make_golden.py``."""
    return json.loads((Path(__file__).resolve().parent / "golden" / "protocols.json").read_text())


@pytest.mark.parametrize("proto,cls", [
    ("ContactForceStrategy", S.GpuHuberContactForce),
    ("FrictionStrategy", S.GpuCoulombReturnMapping),
    ("ContactGeometryStrategy", S.GpuPointToPoint),
    ("ContactGeometryStrategy", S.GpuLineToLineGauss),
    ("ContactGeometryStrategy", S.GpuMortarSegment),
    ("PenaltyStrategy", P.AutoEALPenalty),
    ("PenaltyStrategy", P.ContinuationPenalty),
    ("TimeIntegrationStrategy", D.GpuGeneralizedAlpha),
    ("TimeIntegrationStrategy", D.QuasiStatic),
])
def test_protocol_signatures(proto, cls):
    """Every Protocol method exists with the reference's parameter names, in order."""
    methods = _reference_protocols()[proto]
    assert methods
    for n, want in methods.items():
        got = [q for q in inspect.signature(getattr(cls, n)).parameters if q != "self"]
        assert got[: len(want)] == want, (n, got, want)


def test_geometry_strategy_factory_selection():
    """create_contact_geometry_strategy picks classes as _create_contact_geometry_strategy does:
    use_mortar over line_contact over mode, the mode names, and the options passed on."""
    f = S.create_contact_geometry_strategy
    assert type(f()) is S.GpuPointToPoint
    assert type(f(mode="line_to_line")) is S.GpuLineToLineGauss
    assert type(f(mode="mortar")) is S.GpuMortarSegment
    assert type(f(line_contact=True)) is S.GpuLineToLineGauss
    assert type(f(use_mortar=True, line_contact=True)) is S.GpuMortarSegment
    assert type(f(mode="unknown")) is S.GpuPointToPoint
    g = f(mode="line_to_line", n_gauss=4, auto_gauss=True, exclude_same_layer=False)
    assert (g._n_gauss, g._auto_gauss, g._exclude_same_layer) == (4, True, False)
