"""The oracle against golden vectors produced by the reference itself (CPU)."""

from __future__ import annotations

import warnings

import numpy as np
import pytest

from conftest import golden, golden_csr, rel_err, sparse_rel_err
from oracle import beam as ob
from oracle import contact as oc

SECTION_KEYS = ["E", "G", "A", "Iy", "Iz", "J", "kappa_y", "kappa_z"]


def _section(z, **kw):
    return ob.Section(*(float(z[k]) for k in SECTION_KEYS), **kw)


def test_beam_elements_large_rotations():
    z = golden("beam_elements")
    n = 6 * len(z["X"])
    K, f = ob.assemble_beam(z["X"], z["conn"], z["u"], _section(z))
    assert rel_err(f, z["beam_f"]) < 1e-13
    assert sparse_rel_err(K, golden_csr(z, "beam_K", n)) < 1e-13


def test_beam_vref_and_scf():
    z = golden("beam_elements")
    n = 6 * len(z["X"])
    K, f = ob.assemble_beam(z["X"], z["conn"], z["u"], _section(z, scf=0.25), v_ref=np.array([0.3, -0.2, 0.9]))
    assert rel_err(f, z["beam_f_vref_scf"]) < 1e-13
    assert sparse_rel_err(K, golden_csr(z, "beam_K_vref_scf", n)) < 1e-13


def test_narrowphase_bit_exact():
    z = golden("narrowphase")
    s, t, dist, normal, par = oc.closest_point(z["xA0"], z["xA1"], z["xB0"], z["xB1"])
    for a, b in ((s, z["s"]), (t, z["t"]), (dist, z["dist"]), (normal, z["normal"]), (par, z["parallel"])):
        assert np.array_equal(a, b)


def test_contact_frame_bit_exact():
    z = golden("narrowphase")
    n, t1, t2 = oc.contact_frame(z["normal"], z["prev_t1"], z["prev_n"])
    assert np.array_equal(n, z["n"]) and np.array_equal(t1, z["t1"]) and np.array_equal(t2, z["t2"])


@pytest.mark.parametrize("name", ["strand7", "strand7_nogap", "strand19_slip"])
def test_strand_sequence(name):
    """Detect, active set and Newton iterations, state carried across increments."""
    z = golden(name)
    X, conn, layer = z["X"], z["conn"], z["elem_layer"]
    n = 6 * len(X)
    radii = np.full(len(conn), float(z["radius"]))
    K, f = ob.assemble_beam(X, conn, z["u0"], _section(z))
    assert rel_err(f, z["beam_f"]) < 1e-12
    assert sparse_rel_err(K, golden_csr(z, "beam_K", n)) < 1e-13
    kp, mu, ktr, sd = (float(z[k]) for k in ("k_pen", "mu", "k_t_ratio", "smoothing_delta"))
    table = oc.empty_table()
    for inc in range(int(z["n_incr"])):
        cd = oc.deformed_coords(X, z[f"inc{inc}_u"])
        table, cands, _ = oc.detect(table, cd, conn, radii, elem_layer=layer, exclude_same_layer=True)
        assert np.array_equal(cands, z[f"inc{inc}_candidates"])
        p = f"inc{inc}_detect_"
        for k in ("ea", "eb", "status"):
            assert np.array_equal(table[k], z[p + k])
        table = oc.update_geometry(table, cd)
        p = f"inc{inc}_geom_"
        for k in ("s", "t", "gap", "normal", "status"):
            assert np.array_equal(table[k], z[p + k]), k
        for it in range(int(z["n_iter"])):
            p = f"inc{inc}_it{it}_"
            table, _, _, parts = oc.contact_iteration(table, X, z[p + "u"], z[f"inc{inc}_u_ref"], n, k_pen=kp,
                                                      k_t_ratio=ktr, mu_eff=mu, smoothing_delta=sd)
            assert rel_err(parts["f_n"], z[p + "f_n"]) < 1e-12
            assert rel_err(parts["f_f"], z[p + "f_f"]) < 1e-12
            assert sparse_rel_err(parts["K_n"], golden_csr(z, p + "K_n", n)) < 1e-12
            assert sparse_rel_err(parts["K_f"], golden_csr(z, p + "K_f", n)) < 1e-12
            for k in ("status", "stick"):
                assert np.array_equal(table[k], z[p + k]), k
            for k in ("p_n", "z_t", "q_trial_norm", "k_pen", "k_t", "dissipation"):
                assert rel_err(table[k], z[p + k]) < 1e-12, k


def test_strand_mesh_generator_matches_reference():
    from xkgpu import strand as xs

    z = golden("meshes")
    warnings.simplefilter("ignore")
    for tag, args, kw in (("w7", (7, 2.0, 40.0, 1, 16), dict(gap=-0.01)),
                          ("w19", (19, 1.0, 20.0, 2, 32), dict(gap=0.0)),
                          ("w37", (37, 0.5, 20.0, 2, 48), dict(gap=-0.0025))):
        m = xs.make_strand(*args, **kw)
        assert np.array_equal(m.conn, z[tag + "_conn"])
        # bit-identical on the platform the fixtures were made on; libm may differ elsewhere
        assert rel_err(m.coords, z[tag + "_X"]) < 1e-15
        assert np.array_equal(np.array([w.layer for w in m.wires]), z[tag + "_layer"])


def test_genalpha_oracle_matches_reference():
    """The Generalized-alpha restatement against GeneralizedAlphaProcess's own outputs."""
    from oracle import dynamics as od

    z = golden("genalpha")
    m = z["m"]
    rng = np.random.default_rng(4)
    rng.uniform(1e-9, 1e-6, m.size)  # the fixture's draws, in order
    for rho, tag in ((0.9, "r09"), (0.5, "r05")):
        ga = od.GeneralizedAlpha(m, rho)
        ga.vel = rng.normal(size=m.size)
        ga.acc = rng.normal(size=m.size) * 1e3
        rng.normal(size=m.size)  # u
        for step in range(3):
            p = f"{tag}_s{step}_"
            dt = float(z[p + "dt"])
            assert np.array_equal(ga.predict(z[p + "u"], dt), z[p + "u_pred"])
            ga.correct(z[p + "u1"], None, dt)
            assert np.array_equal(ga.acc, z[p + "acc"]) and np.array_equal(ga.vel, z[p + "vel"])
            assert np.array_equal(ga.effective_residual(z[p + "R"], dt), z[p + "R_eff"])
            assert np.allclose(ga.effective_stiffness_diag(dt), z[p + "K_eff_diag"], rtol=1e-12, atol=0)
            rng.normal(size=m.size)  # u1 noise
            rng.normal(size=m.size)  # R


def test_softplus_law_oracle_matches_reference():
    z = golden("laws")
    p, dp = oc.softplus_normal_law(z["gap"], float(z["k_pen"]), z["lam"], float(z["delta"]))
    assert np.array_equal(p, z["p_n"]) and np.array_equal(dp, z["dp_dg"])


def test_gauss_point_counts_match_reference():
    """auto_n_gauss against _auto_select_n_gauss's own outputs (all three counts and zero-length segments)."""
    z = golden("gauss_points")
    ng = oc.auto_n_gauss(z["xA1"] - z["xA0"], z["xB1"] - z["xB0"])
    assert np.array_equal(ng, z["n_gauss"])
    assert set(np.unique(ng)) == {2, 3, 5}


def test_coating_oracle_matches_reference():
    """Coated wires (Kelvin-Voigt coating with friction): the oracle's coating geometry, forces and
    tangents against KelvinVoigtCoatingProcess's own outputs over two iterations (stick, slip and
    uncompressed pairs whose coating friction history is reset)."""
    z = golden("coating7")
    X, conn, layer = z["X"], z["conn"], z["elem_layer"]
    n = 6 * len(X)
    r, cr = float(z["radius"]), float(z["core_radius"])
    k, c, mu, ktr, dt = (float(z[q]) for q in ("k_coat", "c_coat", "mu_coat", "kt_ratio", "dt"))
    cd = oc.deformed_coords(X, z["u0"])
    table, _, _ = oc.detect(oc.empty_table(), cd, conn, np.full(len(conn), r), elem_layer=layer,
                            exclude_same_layer=True, core_radii=np.full(len(conn), cr))
    for q in ("ea", "eb", "status"):
        assert np.array_equal(table[q], z["detect_" + q])
    table, cc = oc.coating_geometry(table, cd)
    for q in ("s", "t", "gap", "normal", "t1", "status"):
        assert np.array_equal(table[q], z["geom_" + q]), q
    assert np.array_equal(cc, z["geom_cc"])
    cc_prev = 0.8 * cc
    state = {"z_t": np.zeros((len(cc), 2)), "stick": np.ones(len(cc), bool), "q_trial_norm": np.zeros(len(cc)),
             "dissipation": np.zeros(len(cc))}
    u_ref = z["u0"]
    for it in range(int(z["n_iter"])):
        p = f"it{it}_"
        cd = oc.deformed_coords(X, z[p + "u"])
        table, cc = oc.coating_geometry(table, cd, freeze_active_set=True)
        for q in ("s", "t", "gap", "normal", "t1", "t2", "status"):
            assert np.array_equal(table[q], z[p + "pre_" + q]), q
        assert np.array_equal(cc, z[p + "pre_cc"])
        assert rel_err(oc.coating_forces(table, cc, cc_prev, n, k, c, dt), z[p + "f_coat"]) < 1e-12
        assert sparse_rel_err(oc.coating_stiffness(table, cc, n, k, c, dt), golden_csr(z, p + "K_coat", n)) < 1e-12
        f, state = oc.coating_friction(table, cc, state, z[p + "u"], u_ref, n, k, ktr, mu)
        assert rel_err(f, z[p + "f_coat_fric"]) < 1e-12
        assert np.array_equal(state["stick"], z[p + "post_coat_stick"])
        assert rel_err(state["z_t"], z[p + "post_coat_z_t"]) < 1e-12
        assert rel_err(state["q_trial_norm"], z[p + "post_coat_qtn"]) < 1e-12
        assert rel_err(state["dissipation"], z[p + "post_coat_diss"]) < 1e-10
        K = oc.coating_friction_stiffness(table, cc, state, n, k, ktr, mu)
        assert sparse_rel_err(K, golden_csr(z, p + "K_coat_fric", n)) < 1e-12


def test_oracle_broadphase_equals_all_pairs():
    """The grid enumeration returns exactly the pairs whose closed boxes overlap: random boxes of mixed
    sizes, boxes that only touch, duplicates, a degenerate (point) box."""
    rng = np.random.default_rng(9)
    n = 400
    lo = rng.uniform(0.0, 10.0, (n, 3))
    hi = lo + rng.uniform(0.0, 2.0, (n, 3)) * (rng.random((n, 1)) < 0.9)
    lo[1], hi[1] = hi[0], hi[0] + 1.0  # touches box 0 at a corner
    lo[2], hi[2] = lo[3].copy(), hi[3].copy()  # duplicate
    got = oc.aabb_overlap_pairs(lo, hi, chunk=997)
    i, j = np.triu_indices(n, 1)
    ok = np.all(lo[i] <= hi[j], axis=1) & np.all(lo[j] <= hi[i], axis=1)
    want = np.stack([i[ok], j[ok]], axis=1)
    assert np.array_equal(got, want)
    assert [0, 1] in got.tolist() and [2, 3] in got.tolist()
