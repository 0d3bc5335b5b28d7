"""The Strategy classes driven exactly as the reference's Newton loop drives its own.

Per increment: DetectCandidates -> UpdateGeometry; per iteration: UpdateGeometry
(frozen active set) -> HuberContactForce.evaluate -> CoulombReturnMapping.evaluate
-> both tangents.  The golden fixtures hold the reference's outputs of this same
sequence on the same inputs (``tests/golden/make_golden.py``).  Pair states,
candidate and active sets are compared bit for bit where the path is exact
(detection, narrowphase), the rest within 1e-10 relative.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, golden_csr, rel_err, sparse_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from oracle import beam as ob  # noqa: E402
from oracle import contact as oc  # noqa: E402
from xkgpu import strategies as S  # noqa: E402

TOL = 1e-10
EXACT = ("ea", "eb", "s", "t", "gap", "normal", "t1", "t2", "status")


def _arrays(pairs):
    order = sorted(range(len(pairs)), key=lambda i: (pairs[i].elem_a, pairs[i].elem_b))
    st = [pairs[i].state for i in order]
    return {
        "ea": np.array([pairs[i].elem_a for i in order], np.int64),
        "eb": np.array([pairs[i].elem_b for i in order], np.int64),
        "s": np.array([x.s for x in st]), "t": np.array([x.t for x in st]), "gap": np.array([x.gap for x in st]),
        "normal": np.array([x.normal for x in st]).reshape(-1, 3),
        "t1": np.array([x.tangent1 for x in st]).reshape(-1, 3),
        "t2": np.array([x.tangent2 for x in st]).reshape(-1, 3),
        "k_pen": np.array([x.k_pen for x in st]), "k_t": np.array([x.k_t for x in st]),
        "p_n": np.array([x.p_n for x in st]), "z_t": np.array([x.z_t for x in st]).reshape(-1, 2),
        "q_trial_norm": np.array([x.q_trial_norm for x in st]),
        "status": np.array([S._code(x.status) for x in st], np.int8),
        "stick": np.array([x.stick for x in st], bool),
        "dissipation": np.array([x.dissipation for x in st]),
    }


def _check_pairs(got, z, prefix, exact=EXACT):
    a = _arrays(got)
    for k in exact:
        assert np.array_equal(a[k], z[prefix + k]), prefix + k
    for k in ("k_pen", "k_t", "p_n", "z_t", "q_trial_norm", "dissipation"):
        assert rel_err(a[k], z[prefix + k]) < TOL, prefix + k
    assert np.array_equal(a["stick"], z[prefix + "stick"]), prefix + "stick"


@pytest.mark.parametrize("name", ["strand7", "strand7_nogap", "strand19_slip"])
def test_strategies_replay_reference_sequence(name):
    z = golden(name)
    X, conn = z["X"], z["conn"]
    ndof = 6 * len(X)
    r = float(z["radius"])
    k_pen, mu = float(z["k_pen"]), float(z["mu"])
    layer = z["elem_layer"]
    cfg = S.ContactConfig(mu=mu, k_t_ratio=float(z["k_t_ratio"]), exclude_same_layer=True,
                          elem_layer_map={int(e): int(layer[e]) for e in range(len(conn))},
                          smoothing_delta=float(z["smoothing_delta"]))
    mgr = S.ContactManager(config=cfg)
    huber = S.GpuHuberContactForce(ndof, smoothing_delta=float(z["smoothing_delta"]))
    fric = S.GpuCoulombReturnMapping(ndof, k_pen=k_pen, k_t_ratio=float(z["k_t_ratio"]))
    detect, update = S.GpuDetectCandidatesProcess(), S.GpuUpdateGeometryProcess()
    for inc in range(int(z["n_incr"])):
        u = z[f"inc{inc}_u"]
        u_ref = z[f"inc{inc}_u_ref"]
        cdef = X + u.reshape(-1, 6)[:, 0:3]
        det = detect.process(S.DetectCandidatesInput(manager=mgr, node_coords=cdef, connectivity=conn, radii=r))
        mgr = det.manager
        assert np.array_equal(np.array(sorted(det.candidates), np.int64).reshape(-1, 2), z[f"inc{inc}_candidates"])
        assert det.n_pairs == len(mgr.pairs)
        _check_pairs(mgr.pairs, z, f"inc{inc}_detect_")
        ug = update.process(S.UpdateGeometryInput(manager=mgr, node_coords=cdef))
        mgr = ug.manager
        _check_pairs(mgr.pairs, z, f"inc{inc}_geom_")
        assert ug.n_active == int(np.count_nonzero(z[f"inc{inc}_geom_status"]))
        for it in range(int(z["n_iter"])):
            p = f"inc{inc}_it{it}_"
            u = z[p + "u"]
            cdef = X + u.reshape(-1, 6)[:, 0:3]
            ugf = update.process(S.UpdateGeometryInput(manager=mgr, node_coords=cdef, freeze_active_set=True))
            mgr.pairs[:] = ugf.manager.pairs
            fn, rn = huber.evaluate(u, mgr, k_pen)
            ff, rf = fric.evaluate(u, mgr.pairs, mu, u_ref=u_ref)
            Kn = huber.tangent(u, mgr, k_pen)
            Kf = fric.tangent(u, mgr.pairs, mu)
            assert rel_err(fn, z[p + "f_n"]) < TOL
            assert rel_err(ff, z[p + "f_f"]) < TOL
            # per-pair residuals follow the pair-list order; the reference's first list is in the
            # iteration order of a Python set, ours sorted by (elem_a, elem_b): compare as multisets
            assert rn.shape == z[p + "res_n"].shape and rel_err(np.sort(rn), np.sort(z[p + "res_n"])) < TOL
            # the friction residual max(0, |q| - mu p_n) of a sliding pair is rounding noise of |q| ~ mu p_n:
            # compare on the scale of mu p_n
            scale = max(mu * float(np.max(z[p + "p_n"], initial=0.0)), 1e-300)
            assert rf.shape == z[p + "res_f"].shape
            assert np.max(np.abs(np.sort(rf) - np.sort(z[p + "res_f"])), initial=0.0) <= TOL * scale
            assert sparse_rel_err(Kn, golden_csr(z, p + "K_n", ndof)) < TOL
            assert sparse_rel_err(Kf, golden_csr(z, p + "K_f", ndof)) < TOL
            _check_pairs(mgr.pairs, z, p, exact=("ea", "eb", "s", "t", "gap", "normal", "t1", "t2", "status"))
            assert bool(fric.friction_tangents) == bool(np.any(z[p + "p_n"] > 0))


def test_point_to_point_detect_and_jacobian():
    """PointToPoint.detect (shared-node exclusion, no prescreen, g_on = g_off = 0) and its Jacobian."""
    z = golden("strand7")
    X, conn = z["X"], z["conn"]
    u = z["inc0_u"]
    cdef = X + u.reshape(-1, 6)[:, 0:3]
    r = float(z["radius"])
    ptp = S.GpuPointToPoint(exclude_same_layer=True)
    pairs = ptp.detect(cdef, conn, r)
    radii = np.full(len(conn), r)
    lo, hi = oc.segment_aabbs(cdef, conn, radii)
    raw = oc.aabb_overlap_pairs(lo, hi)
    cands = oc.filter_candidates(raw, cdef, conn, radii, midpoint_prescreening=False)
    tab = oc.merge_candidates(oc.empty_table(), cands, conn, radii)
    tab = oc.update_geometry(tab, cdef, g_on=0.0, g_off=0.0)
    a = _arrays(pairs)
    for k in ("ea", "eb", "s", "t", "gap", "normal", "t1", "t2", "status"):
        assert np.array_equal(a[k], tab[k]), k
    assert ptp.compute_gap(pairs[0], cdef) == pairs[0].state.gap
    # the geometry update moves with the nodes
    cdef2 = cdef + 1e-3 * np.sin(np.arange(cdef.size)).reshape(cdef.shape)
    ptp.update_geometry(pairs, cdef2)
    tab2 = oc.update_geometry(tab, cdef2, g_on=0.0, g_off=0.0)
    a = _arrays(pairs)
    for k in ("s", "t", "gap", "normal", "t1", "t2", "status"):
        assert np.array_equal(a[k], tab2[k]), k
    G, act = ptp.build_constraint_jacobian(pairs, 6 * len(X))
    order = sorted(range(len(pairs)), key=lambda i: (pairs[i].elem_a, pairs[i].elem_b))
    assert order == list(range(len(pairs)))
    Ge, acte = oc.constraint_jacobian(tab2, 6 * len(X))
    assert act == acte
    assert sparse_rel_err(G, Ge) < 1e-15


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_cr_beam_assembler(precision, tol):
    z = golden("beam_elements")
    sec = {k: float(z[k]) for k in ("E", "G", "A", "Iy", "Iz", "J", "kappa_y", "kappa_z")}
    asm = S.GpuCRBeamAssembler(z["X"], z["conn"], sec["E"], sec["G"], sec["A"], sec["Iy"], sec["Iz"], sec["J"],
                               sec["kappa_y"], sec["kappa_z"], precision=precision)
    n = 6 * len(z["X"])
    assert rel_err(asm.assemble_internal_force(z["u"]), z["beam_f"]) < tol
    assert sparse_rel_err(asm.assemble_tangent(z["u"]), golden_csr(z, "beam_K", n)) < tol
    # updated Lagrangian: move the reference by a converged increment, then assemble the next one
    X0 = np.asarray(z["X"], dtype=float)
    du = 0.2 * np.asarray(z["u"], dtype=float)
    asm.checkpoint()
    asm.update_reference(du)
    X1 = X0 + du.reshape(-1, 6)[:, 0:3]
    assert np.allclose(asm.coords_ref, X1, rtol=0, atol=1e-14)
    u2 = 0.5 * np.asarray(z["u"], dtype=float)
    Ke, fe = ob.assemble_beam(X1, z["conn"], u2, ob.Section(**sec, scf=None))
    assert rel_err(asm.assemble_internal_force(u2), fe) < tol
    assert sparse_rel_err(asm.assemble_tangent(u2), Ke) < tol
    assert np.array_equal(asm.get_total_displacement(u2), du + u2)
    asm.rollback()
    assert np.array_equal(asm.coords_ref, X0)
    assert rel_err(asm.assemble_internal_force(z["u"]), z["beam_f"]) < tol
    M = asm.assemble_mass(7.85e-9)
    me = ob.lumped_mass_diag(X0, z["conn"], 7.85e-9, ob.Section(**sec, scf=None))
    assert rel_err(M.diagonal(), me) < 1e-14
    with pytest.raises(NotImplementedError):
        asm.assemble_mass(7.85e-9, lumped=False)


def test_smooth_normal_law_matches_reference():
    z = golden("laws")
    p, dp = S.smooth_normal_force(z["gap"], float(z["k_pen"]), z["lam"], delta=float(z["delta"]))
    assert rel_err(p, z["p_n"]) < 1e-14 and rel_err(dp, z["dp_dg"]) < 1e-14
    # the cut-offs and the lambda-free form
    g = np.linspace(-1e-2, 1e-2, 2001)
    p0, d0 = S.smooth_normal_force(g, 1e5, None, delta=1e-4)
    pe, de = oc.softplus_normal_law(g, 1e5, np.zeros_like(g), 1e-4)
    assert rel_err(p0, pe) < 1e-14 and rel_err(d0, de) < 1e-14


def test_line_to_line_gauss_points_and_geometry():
    """Gauss-point counts on the GPU equal the reference's (golden), and the line-to-line and mortar
    strategies update the geometry exactly as point-to-point, setting _n_gauss where a pair has it."""
    z = golden("gauss_points")
    n = z["xA0"].shape[0]
    X = np.concatenate([z["xA0"], z["xA1"], z["xB0"], z["xB1"]])
    Pair, State, _ = S.pair_types()
    pairs = [Pair(elem_a=2 * i, elem_b=2 * i + 1, nodes_a=np.array([i, n + i]), nodes_b=np.array([2 * n + i, 3 * n + i]),
                  state=State(), radius_a=0.1, radius_b=0.1) for i in range(n)]
    ng = S.pair_gauss_points(pairs, X)
    assert np.array_equal(ng, z["n_gauss"])
    assert np.array_equal(ng, oc.auto_n_gauss(z["xA1"] - z["xA0"], z["xB1"] - z["xB0"]))

    import dataclasses

    # a mutable pair type that carries the attribute the reference checks for
    spec = []
    for f in dataclasses.fields(Pair):
        if f.default is not dataclasses.MISSING:
            spec.append((f.name, f.type, dataclasses.field(default=f.default)))
        elif f.default_factory is not dataclasses.MISSING:
            spec.append((f.name, f.type, dataclasses.field(default_factory=f.default_factory)))
        else:
            spec.append((f.name, f.type))
    WithGauss = dataclasses.make_dataclass("WithGauss", spec + [("_n_gauss", int, dataclasses.field(default=0))])
    tagged = [WithGauss(**{f.name: getattr(p, f.name) for f in dataclasses.fields(p)}) for p in pairs]
    ptp, l2l = list(pairs), list(tagged)
    S.GpuPointToPoint().update_geometry(ptp, X)
    S.create_contact_geometry_strategy(line_contact=True, auto_gauss=True).update_geometry(l2l, X)
    mortar = list(pairs)
    S.create_contact_geometry_strategy(use_mortar=True).update_geometry(mortar, X)
    for a, b, c in zip(ptp, l2l, mortar):
        for k in ("s", "t", "gap"):
            assert getattr(a.state, k) == getattr(b.state, k) == getattr(c.state, k)
        assert np.array_equal(a.state.normal, b.state.normal) and np.array_equal(a.state.tangent1, c.state.tangent1)
    assert np.array_equal(np.array([p._n_gauss for p in l2l]), z["n_gauss"])


def test_coating_strategy_replays_reference():
    """GpuKelvinVoigtCoating and the coated geometry update driven as the reference's solver drives
    KelvinVoigtCoatingProcess, against its recorded outputs (tests/golden/coating7.npz)."""
    import dataclasses

    z = golden("coating7")
    X, conn, layer = z["X"], z["conn"], z["elem_layer"]
    ndof = 6 * len(X)
    r, cr = float(z["radius"]), float(z["core_radius"])
    k, c, mu, ktr, dt = (float(z[q]) for q in ("k_coat", "c_coat", "mu_coat", "kt_ratio", "dt"))
    cfg = S.ContactConfig(exclude_same_layer=True, elem_layer_map={int(e): int(layer[e]) for e in range(len(conn))},
                          coating_stiffness=k, coating_damping=c, coating_mu=mu, coating_k_t_ratio=ktr)
    mgr = S.ContactManager(config=cfg)
    cdef = X + z["u0"].reshape(-1, 6)[:, 0:3]
    det = S.GpuDetectCandidatesProcess().process(
        S.DetectCandidatesInput(manager=mgr, node_coords=cdef, connectivity=conn, radii=r, core_radii=cr))
    mgr = det.manager
    mgr = S.GpuUpdateGeometryProcess().process(S.UpdateGeometryInput(manager=mgr, node_coords=cdef)).manager
    _check_geometry(mgr.pairs, z, "geom_")
    pairs = [S._evolve(p, coating_compression_prev=0.8 * p.state.coating_compression) for p in mgr.pairs]
    mgr = dataclasses.replace(mgr, pairs=pairs)
    kv = S.create_coating_strategy(coating_stiffness=k)
    assert isinstance(kv, S.GpuKelvinVoigtCoating)
    u_ref = z["u0"]
    for it in range(int(z["n_iter"])):
        p = f"it{it}_"
        u = z[p + "u"]
        cdef = X + u.reshape(-1, 6)[:, 0:3]
        mgr = S.GpuUpdateGeometryProcess().process(
            S.UpdateGeometryInput(manager=mgr, node_coords=cdef, freeze_active_set=True)).manager
        _check_geometry(mgr.pairs, z, p + "pre_")
        pl = list(mgr.pairs)
        assert rel_err(kv.forces(pl, cdef, cfg, dt), z[p + "f_coat"]) < TOL
        assert sparse_rel_err(kv.stiffness(pl, cdef, cfg, ndof, dt), golden_csr(z, p + "K_coat", ndof)) < TOL
        assert rel_err(kv.friction_forces(pl, cdef, cfg, u, u_ref), z[p + "f_coat_fric"]) < TOL
        co = _coating(pl)
        assert np.array_equal(co["stick"], z[p + "post_coat_stick"])
        for q, g in (("z_t", "coat_z_t"), ("qtn", "coat_qtn"), ("diss", "coat_diss")):
            assert rel_err(co[q], z[p + "post_" + g]) < TOL, q
        K = kv.friction_stiffness(pl, cdef, cfg, ndof)
        assert sparse_rel_err(K, golden_csr(z, p + "K_coat_fric", ndof)) < TOL
        mgr = dataclasses.replace(mgr, pairs=pl)
    none = S.create_coating_strategy(coating_stiffness=0.0)
    assert not np.any(none.forces(pl, cdef, cfg, dt)) and none.stiffness(pl, cdef, cfg, ndof, dt).nnz == 0


def _coating(pairs):
    order = sorted(range(len(pairs)), key=lambda i: (pairs[i].elem_a, pairs[i].elem_b))
    st = [pairs[i].state for i in order]
    return {"cc": np.array([x.coating_compression for x in st]),
            "z_t": np.array([x.coating_z_t for x in st]).reshape(-1, 2),
            "stick": np.array([x.coating_stick for x in st], bool),
            "qtn": np.array([x.coating_q_trial_norm for x in st]),
            "diss": np.array([x.coating_dissipation for x in st])}


def _check_geometry(pairs, z, prefix):
    a = _arrays(pairs)
    for q in ("ea", "eb", "s", "t", "gap", "normal", "t1", "t2", "status"):
        assert np.array_equal(a[q], z[prefix + q]), prefix + q
    assert np.array_equal(_coating(pairs)["cc"], z[prefix + "cc"])
