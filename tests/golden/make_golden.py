"""Generate the golden fixtures by running the xkep-cae reference itself.

Run in a container that holds the reference source tree:

    python tests/golden/make_golden.py /path/to/xkep-cae [case ...]

The reference is imported read-only (no bytecode written, its process report
hook switched off) and driven through its own public functions on seeded
strand states.  Each fixture is a compressed ``.npz`` next to this script.
Pair data are stored sorted by ``(elem_a, elem_b)`` so that they can be
compared with any pair-table order.
"""

from __future__ import annotations

import math
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _import_reference(root: str):
    sys.dont_write_bytecode = True
    os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
    sys.path.insert(0, root)
    import warnings

    warnings.simplefilter("ignore")
    from xkep_cae.core.diagnostics import ProcessExecutionLog

    log = ProcessExecutionLog.instance()
    log.enabled = False
    log._report_on_exit = False
    import xkep_cae.contact._manager_process as mp
    import xkep_cae.contact.contact_force.strategy as cf
    import xkep_cae.contact.friction.strategy as fs
    import xkep_cae.contact.geometry._compute as gc
    import xkep_cae.contact.geometry.strategy as gs
    import xkep_cae.contact.penalty.law_normal as ln
    import xkep_cae.contact.penalty.strategy as ps
    import xkep_cae.contact._contact_pair as cp
    import xkep_cae.elements._beam_assembly as ba
    import xkep_cae.elements._beam_section as bs
    import xkep_cae.mesh._twisted_wire as tw
    import xkep_cae.time_integration.strategy as ti

    return dict(mp=mp, cf=cf, fs=fs, gc=gc, gs=gs, ln=ln, ps=ps, cp=cp, ba=ba, bs=bs, tw=tw, ti=ti)


def _section(R, d, E=2.0e5, nu=0.3):
    sec = R["bs"].BeamSectionInput.circle(d)
    kap = sec.cowper_kappa_y(nu)
    return dict(E=E, G=E / (2.0 * (1.0 + nu)), A=sec.A, Iy=sec.Iy, Iz=sec.Iz, J=sec.J,
                kappa_y=kap, kappa_z=kap)


def _pairs_to_arrays(pairs):
    order = sorted(range(len(pairs)), key=lambda i: (pairs[i].elem_a, pairs[i].elem_b))
    ps = [pairs[i] for i in order]
    st = [p.state for p in ps]
    return {
        "ea": np.array([p.elem_a for p in ps], dtype=np.int64),
        "eb": np.array([p.elem_b for p in ps], dtype=np.int64),
        "s": np.array([x.s for x in st]), "t": np.array([x.t for x in st]),
        "gap": np.array([x.gap for x in st]),
        "normal": np.array([x.normal for x in st]).reshape(-1, 3),
        "t1": np.array([x.tangent1 for x in st]).reshape(-1, 3),
        "t2": np.array([x.tangent2 for x in st]).reshape(-1, 3),
        "k_pen": np.array([x.k_pen for x in st]), "k_t": np.array([x.k_t for x in st]),
        "p_n": np.array([x.p_n for x in st]),
        "z_t": np.array([x.z_t for x in st]).reshape(-1, 2),
        "q_trial_norm": np.array([x.q_trial_norm for x in st]),
        "status": np.array([x.status.value for x in st], dtype=np.int8),
        "stick": np.array([x.stick for x in st], dtype=bool),
        "dissipation": np.array([x.dissipation for x in st]),
    }


def _csr(prefix, K, out):
    K = K.tocsr()
    K.sum_duplicates()
    out[prefix + "_data"] = K.data
    out[prefix + "_indices"] = K.indices.astype(np.int64)
    out[prefix + "_indptr"] = K.indptr.astype(np.int64)


def strand_case(R, name, *, n_wires, d, pitch, n_pitches, n_el, gap_frac, seed, mu, k_t_ratio=0.5,
                smoothing_delta=0.0, sigma_pos_frac=1e-3, sigma_rot=1e-3, n_iter=2, n_incr=2,
                step_frac=3e-4):
    """Beam + contact sequence: (detect, active set, ``n_iter`` Newton iterations) x ``n_incr``."""
    mesh = R["tw"]._make_twisted_wire_mesh(n_wires, d, pitch, 0.0, n_el, n_pitches=n_pitches,
                                           gap=gap_frac * d)
    X = mesh.node_coords.copy()
    conn = mesh.connectivity.astype(np.int64)
    layer = np.array([mesh.strand_infos[e // n_el].layer for e in range(len(conn))], dtype=np.int32)
    sec = _section(R, d)
    ndof = 6 * len(X)
    rng = np.random.default_rng(seed)
    u = np.zeros(ndof)
    uu = u.reshape(-1, 6)
    uu[:, 0:3] = rng.normal(0.0, sigma_pos_frac * d, (len(X), 3))
    uu[:, 3:6] = rng.normal(0.0, sigma_rot, (len(X), 3))
    L_mean = float(np.mean(np.linalg.norm(X[conn[:, 1]] - X[conn[:, 0]], axis=1)))
    k_pen = R["ps"].AutoEALPenalty(sec["E"], sec["A"], L_mean, scale=1e3).compute_k_pen(0, 1)
    r = d / 2.0
    cfg = R["cp"]._ContactConfigInput(mu=mu, k_t_ratio=k_t_ratio, exclude_same_layer=True,
                                      elem_layer_map={int(e): int(layer[e]) for e in range(len(conn))},
                                      smoothing_delta=smoothing_delta)
    mgr = R["cp"]._ContactManagerInput(config=cfg)
    out = dict(X=X, conn=conn, elem_layer=layer, radius=np.array(r), k_pen=np.array(k_pen),
               mu=np.array(mu), k_t_ratio=np.array(k_t_ratio), smoothing_delta=np.array(smoothing_delta),
               n_iter=np.array(n_iter), n_incr=np.array(n_incr), **{k: np.array(v) for k, v in sec.items()})
    # beam at the seeded state
    K, f = R["ba"].assemble_cr_beam3d(X, conn, u, sec["E"], sec["G"], sec["A"], sec["Iy"], sec["Iz"],
                                      sec["J"], sec["kappa_y"], sec["kappa_z"])
    out["u0"] = u.copy()
    out["beam_f"] = f
    _csr("beam_K", K, out)
    huber = R["cf"].HuberContactForceProcess(ndof, smoothing_delta=smoothing_delta)
    fric = R["fs"].CoulombReturnMappingProcess(ndof, k_pen=k_pen, k_t_ratio=k_t_ratio)
    u_ref = np.zeros(ndof)
    step_rng = np.random.default_rng(seed + 1000)
    for inc in range(n_incr):
        coords_def = X + u.reshape(-1, 6)[:, 0:3]
        det = R["mp"].DetectCandidatesProcess().process(
            R["mp"].DetectCandidatesInput(manager=mgr, node_coords=coords_def, connectivity=conn, radii=r))
        mgr = det.manager
        cands = np.array(sorted(det.candidates), dtype=np.int64).reshape(-1, 2)
        out[f"inc{inc}_u"] = u.copy()
        out[f"inc{inc}_u_ref"] = u_ref.copy()
        out[f"inc{inc}_candidates"] = cands
        for k, v in _pairs_to_arrays(mgr.pairs).items():
            out[f"inc{inc}_detect_{k}"] = v
        ug = R["mp"].UpdateGeometryProcess().process(R["mp"].UpdateGeometryInput(manager=mgr, node_coords=coords_def))
        mgr = ug.manager
        for k, v in _pairs_to_arrays(mgr.pairs).items():
            out[f"inc{inc}_geom_{k}"] = v
        for it in range(n_iter):
            du = step_rng.normal(0.0, step_frac * d, (len(X), 3))
            u = u.copy()
            u.reshape(-1, 6)[:, 0:3] += du
            cdef = X + u.reshape(-1, 6)[:, 0:3]
            ugf = R["mp"].UpdateGeometryProcess().process(
                R["mp"].UpdateGeometryInput(manager=mgr, node_coords=cdef, freeze_active_set=True))
            mgr.pairs[:] = ugf.manager.pairs
            fn, rn = huber.evaluate(u, mgr, k_pen)
            ff, rf = fric.evaluate(u, mgr.pairs, mu, u_ref=u_ref)
            Kn = huber.tangent(u, mgr, k_pen)
            Kf = fric.tangent(u, mgr.pairs, mu)
            p = f"inc{inc}_it{it}_"
            out[p + "u"] = u.copy()
            out[p + "f_n"] = fn
            out[p + "f_f"] = ff
            out[p + "res_n"] = rn
            out[p + "res_f"] = rf
            _csr(p + "K_n", Kn, out)
            _csr(p + "K_f", Kf, out)
            for k, v in _pairs_to_arrays(mgr.pairs).items():
                out[p + k] = v
        u_ref = u.copy()
        # next increment starts from a perturbed state
        u = u.copy()
        u.reshape(-1, 6)[:, 0:3] += step_rng.normal(0.0, 2 * step_frac * d, (len(X), 3))
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, "nodes", len(X), "elems", len(conn), "pairs", len(mgr.pairs))


def narrowphase_case(R, name, seed=7, n=2000):
    """Segment pairs of many shapes through the batched closest point and frame."""
    rng = np.random.default_rng(seed)
    xA0 = rng.normal(size=(n, 3))
    dA = rng.normal(size=(n, 3))
    xB0 = xA0 + rng.normal(size=(n, 3)) * rng.uniform(0.01, 2.0, (n, 1))
    dB = rng.normal(size=(n, 3))
    k = n // 8
    dB[:k] = dA[:k] * rng.uniform(-2, 2, (k, 1))                    # parallel
    dB[k:2 * k] = dA[k:2 * k] * (1 + 1e-7 * rng.normal(size=(k, 1)))  # nearly parallel
    dA[2 * k:2 * k + 20] = 0.0                                       # degenerate A
    dB[2 * k + 20:2 * k + 40] = 0.0                                  # degenerate B
    xB0[2 * k + 40:2 * k + 60] = xA0[2 * k + 40:2 * k + 60]          # touching start points
    dB[2 * k + 40:2 * k + 60] = dA[2 * k + 40:2 * k + 60]            # identical segments
    xA1, xB1 = xA0 + dA, xB0 + dB
    s, t, pa, pb, dist, normal, par = R["gc"]._closest_point_segments_batch(xA0, xA1, xB0, xB1)
    prev_n = rng.normal(size=(n, 3))
    prev_n /= np.linalg.norm(prev_n, axis=1, keepdims=True)
    prev_t1 = rng.normal(size=(n, 3))
    prev_t1 -= np.sum(prev_t1 * prev_n, axis=1, keepdims=True) * prev_n
    prev_t1 /= np.linalg.norm(prev_t1, axis=1, keepdims=True)
    prev_n[-200:] = 0.0           # no previous normal: Gram-Schmidt route
    prev_t1[-100:] = 0.0          # no previous tangent: seeded route
    prev_n[:50] = normal[:50]     # unchanged normal: no transport rotation
    has_t1 = np.sqrt(np.einsum("ij,ij->i", prev_t1, prev_t1)) > 1e-10
    has_n = np.sqrt(np.einsum("ij,ij->i", prev_n, prev_n)) > 1e-10
    nn, t1, t2 = R["gc"]._build_contact_frame_batch(normal, prev_tangent1s=prev_t1, prev_normals=prev_n,
                                                     has_prev_mask=has_t1, has_prev_n_mask=has_n)
    np.savez_compressed(HERE / f"{name}.npz", xA0=xA0, xA1=xA1, xB0=xB0, xB1=xB1, s=s, t=t, dist=dist,
                        normal=normal, parallel=par, prev_n=prev_n, prev_t1=prev_t1, n=nn, t1=t1, t2=t2)
    print(name, n)


def beam_case(R, name, seed=3, n=64):
    """Isolated elements with large rotations and arbitrary orientations."""
    rng = np.random.default_rng(seed)
    X = np.zeros((2 * n, 3))
    X[0::2] = rng.normal(size=(n, 3))
    X[1::2] = X[0::2] + rng.normal(size=(n, 3)) * 0.7
    X[1:8:2] = X[0:8:2] + np.array([0.0, 0.0, 1.3])       # axis-aligned elements
    conn = np.stack([np.arange(0, 2 * n, 2), np.arange(1, 2 * n, 2)], axis=1)
    u = np.zeros(12 * n)
    uu = u.reshape(-1, 6)
    uu[:, 0:3] = rng.normal(size=(2 * n, 3)) * 0.05
    uu[:, 3:6] = rng.normal(size=(2 * n, 3)) * rng.uniform(1e-6, 1.5, (2 * n, 1))
    uu[0:4, 3:6] = 0.0                                    # zero rotation
    sec = _section(R, 0.3)
    K, f = R["ba"].assemble_cr_beam3d(X, conn, u, sec["E"], sec["G"], sec["A"], sec["Iy"], sec["Iz"],
                                      sec["J"], sec["kappa_y"], sec["kappa_z"])
    out = dict(X=X, conn=conn, u=u, beam_f=f, **{k: np.array(v) for k, v in sec.items()})
    _csr("beam_K", K, out)
    # the same elements with a fixed reference vector and shear-slenderness compensation
    K2, f2 = R["ba"].assemble_cr_beam3d(X, conn, u, sec["E"], sec["G"], sec["A"], sec["Iy"], sec["Iz"],
                                        sec["J"], sec["kappa_y"], sec["kappa_z"],
                                        v_ref=np.array([0.3, -0.2, 0.9]), scf=0.25)
    out["beam_f_vref_scf"] = f2
    _csr("beam_K_vref_scf", K2, out)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, n)


def mesh_case(R, name):
    out = {}
    for tag, args, kw in (("w7", (7, 2.0, 40.0, 0.0, 16), dict(n_pitches=1, gap=-0.01)),
                          ("w19", (19, 1.0, 20.0, 0.0, 32), dict(n_pitches=2, gap=0.0)),
                          ("w37", (37, 0.5, 20.0, 0.0, 48), dict(n_pitches=2, gap=-0.0025))):
        m = R["tw"]._make_twisted_wire_mesh(*args, **kw)
        out[tag + "_X"] = m.node_coords
        out[tag + "_conn"] = m.connectivity.astype(np.int64)
        out[tag + "_layer"] = np.array([s.layer for s in m.strand_infos], dtype=np.int64)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name)


def laws_case(R, name):
    g = np.linspace(-2e-3, 2e-3, 101)
    lam = np.linspace(0.0, 5.0, 101)
    p, dp = R["ln"]._evaluate_smooth_normal_force_vectorized(g, 1e4, lam, delta=1e-4)
    np.savez_compressed(HERE / f"{name}.npz", gap=g, lam=lam, k_pen=np.array(1e4), delta=np.array(1e-4),
                        p_n=p, dp_dg=dp)
    print(name)


def genalpha_case(R, name, seed=4, n=600):
    """GeneralizedAlphaProcess with a lumped mass: predict / correct / effective terms over three steps."""
    import scipy.sparse as sp

    ti = R["ti"]
    rng = np.random.default_rng(seed)
    m = rng.uniform(1e-9, 1e-6, n)
    out = {"m": m}
    for rho, tag in ((0.9, "r09"), (0.5, "r05")):
        ga = ti.GeneralizedAlphaProcess(sp.diags(m, format="csr"), rho_inf=rho)
        ga.set_initial_state(velocity=rng.normal(size=n), acceleration=rng.normal(size=n) * 1e3)
        u = rng.normal(size=n) * 1e-3
        K = sp.random(n, n, density=0.01, random_state=seed, format="csr") + sp.eye(n, format="csr")
        for step, dt in enumerate((1e-4, 2e-4, 1e-4)):
            p = f"{tag}_s{step}_"
            out[p + "u"] = u.copy()
            out[p + "dt"] = np.array(dt)
            out[p + "u_pred"] = ga.predict(u, dt)
            u1 = out[p + "u_pred"] + rng.normal(size=n) * 1e-6
            out[p + "u1"] = u1
            ga.correct(u1, u1 - out[p + "u_pred"], dt)
            out[p + "acc"], out[p + "vel"] = ga.acc.copy(), ga.vel.copy()
            R_in = rng.normal(size=n)
            out[p + "R"] = R_in
            out[p + "R_eff"] = ga.effective_residual(R_in, dt)
            out[p + "K_eff_diag"] = ga.effective_stiffness(K, dt).diagonal() - K.diagonal()
            u = u1
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name)


def _coating_arrays(pairs):
    order = sorted(range(len(pairs)), key=lambda i: (pairs[i].elem_a, pairs[i].elem_b))
    st = [pairs[i].state for i in order]
    return {
        "cc": np.array([x.coating_compression for x in st]),
        "cc_prev": np.array([x.coating_compression_prev for x in st]),
        "coat_z_t": np.array([x.coating_z_t for x in st]).reshape(-1, 2),
        "coat_stick": np.array([x.coating_stick for x in st], dtype=bool),
        "coat_qtn": np.array([x.coating_q_trial_norm for x in st]),
        "coat_diss": np.array([x.coating_dissipation for x in st]),
        "core_a": np.array([pairs[i].core_radius_a for i in order]),
        "core_b": np.array([pairs[i].core_radius_b for i in order]),
    }


def coating_case(R, name, *, n_wires=7, d=2.0, pitch=40.0, n_el=16, gap_frac=-0.005, core_frac=0.9, seed=21,
                 k_coat=1e4, c_coat=50.0, mu_coat=0.2, kt_ratio=0.5, dt=0.1, n_iter=2, step_frac=5e-3):
    """Kelvin-Voigt coating: detection with core radii, the coating geometry (active set and frozen),
    then per iteration forces, stiffness, friction forces (state update) and friction stiffness."""
    import xkep_cae.contact.coating.strategy as cs

    mesh = R["tw"]._make_twisted_wire_mesh(n_wires, d, pitch, 0.0, n_el, n_pitches=1, gap=gap_frac * d)
    X = mesh.node_coords.copy()
    conn = mesh.connectivity.astype(np.int64)
    layer = np.array([mesh.strand_infos[e // n_el].layer for e in range(len(conn))], dtype=np.int32)
    ndof = 6 * len(X)
    r = d / 2.0
    rng = np.random.default_rng(seed)
    u = np.zeros(ndof)
    u.reshape(-1, 6)[:, 0:3] = rng.normal(0.0, 1e-3 * d, (len(X), 3))
    cfg = R["cp"]._ContactConfigInput(exclude_same_layer=True,
                                      elem_layer_map={int(e): int(layer[e]) for e in range(len(conn))},
                                      coating_stiffness=k_coat, coating_damping=c_coat, coating_mu=mu_coat,
                                      coating_k_t_ratio=kt_ratio)
    mgr = R["cp"]._ContactManagerInput(config=cfg)
    out = dict(X=X, conn=conn, elem_layer=layer, radius=np.array(r), core_radius=np.array(core_frac * r),
               k_coat=np.array(k_coat), c_coat=np.array(c_coat), mu_coat=np.array(mu_coat),
               kt_ratio=np.array(kt_ratio), dt=np.array(dt), n_iter=np.array(n_iter), u0=u.copy())
    cdef = X + u.reshape(-1, 6)[:, 0:3]
    det = R["mp"].DetectCandidatesProcess().process(
        R["mp"].DetectCandidatesInput(manager=mgr, node_coords=cdef, connectivity=conn, radii=r,
                                      core_radii=core_frac * r))
    mgr = det.manager
    for k, v in _pairs_to_arrays(mgr.pairs).items():
        out["detect_" + k] = v
    ug = R["mp"].UpdateGeometryProcess().process(R["mp"].UpdateGeometryInput(manager=mgr, node_coords=cdef))
    mgr = ug.manager
    for k, v in {**_pairs_to_arrays(mgr.pairs), **_coating_arrays(mgr.pairs)}.items():
        out["geom_" + k] = v
    # a previous-step compression for the dashpot term (process.py:539-545 sets it at step ends)
    mgr.pairs[:] = [R["cp"]._evolve_pair(p, state=R["cp"]._evolve_state(
        p.state, coating_compression_prev=0.8 * p.state.coating_compression)) for p in mgr.pairs]
    kv = cs.KelvinVoigtCoatingProcess()
    u_ref = u.copy()
    step_rng = np.random.default_rng(seed + 1)
    for it in range(n_iter):
        u = u.copy()
        u.reshape(-1, 6)[:, 0:3] += step_rng.normal(0.0, step_frac * d, (len(X), 3))
        cdef = X + u.reshape(-1, 6)[:, 0:3]
        ugf = R["mp"].UpdateGeometryProcess().process(
            R["mp"].UpdateGeometryInput(manager=mgr, node_coords=cdef, freeze_active_set=True))
        mgr.pairs[:] = ugf.manager.pairs
        p = f"it{it}_"
        out[p + "u"] = u.copy()
        for k, v in {**_pairs_to_arrays(mgr.pairs), **_coating_arrays(mgr.pairs)}.items():
            out[p + "pre_" + k] = v
        out[p + "f_coat"] = kv.forces(mgr.pairs, cdef, cfg, dt)
        _csr(p + "K_coat", kv.stiffness(mgr.pairs, cdef, cfg, ndof, dt), out)
        out[p + "f_coat_fric"] = kv.friction_forces(mgr.pairs, cdef, cfg, u, u_ref)
        _csr(p + "K_coat_fric", kv.friction_stiffness(mgr.pairs, cdef, cfg, ndof), out)
        for k, v in _coating_arrays(mgr.pairs).items():
            out[p + "post_" + k] = v
    np.savez_compressed(HERE / f"{name}.npz", **out)
    cc = out["geom_cc"]
    print(name, "pairs", len(mgr.pairs), "compressed", int(np.sum(cc > 0)),
          "slip", int(np.sum(~out[f"it{n_iter - 1}_post_coat_stick"])))


def gauss_case(R, name, seed=11, n=1200):
    """Gauss-point counts of segment pairs at every angle (line-to-line / mortar auto_gauss)."""
    rng = np.random.default_rng(seed)
    dA = rng.normal(size=(n, 3))
    ang = rng.uniform(0.0, np.pi, n)
    # a unit vector at angle ang to dA, in a random plane through dA
    a = dA / np.linalg.norm(dA, axis=1, keepdims=True)
    w = rng.normal(size=(n, 3))
    w -= np.sum(w * a, axis=1, keepdims=True) * a
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    dB = (np.cos(ang)[:, None] * a + np.sin(ang)[:, None] * w) * rng.uniform(0.1, 3.0, (n, 1))
    dA[:10] = 0.0            # zero-length A
    dB[10:20] = 0.0          # zero-length B
    xA0 = rng.normal(size=(n, 3))
    xB0 = rng.normal(size=(n, 3))
    ng = np.array([R["gc"]._auto_select_n_gauss(dA[i], dB[i]) for i in range(n)])
    np.savez_compressed(HERE / f"{name}.npz", xA0=xA0, xA1=xA0 + dA, xB0=xB0, xB1=xB0 + dB, n_gauss=ng)
    print(name, n, np.bincount(ng))


def solve_case(R, name, *, n_wires=7, d=2.0, pitch=40.0, n_el=16, kappa=0.0, twist=0.0, t_total=1e-3, mu=0.1,
               kpen_scale=1e3, smoothing_delta=0.0, dt_max_fraction=0.1, rho=7.85e-9, rho_inf=0.9):
    """One run of the reference's own ``ContactFrictionProcess`` (``contact/solver/process.py:139-674``)
    on a strand clamped at z = 0 whose z = L ends are driven to a prescribed end state: the section
    of a circular arc of curvature ``kappa`` (bending about x) or a rigid twist by ``twist`` about
    the strand axis, ramped over ``t_total`` with lumped mass and Generalized-alpha.  Records the
    inputs, every Newton call's residual history (retries included) and the displacements of every
    converged increment."""
    import importlib

    data = importlib.import_module("xkep_cae.core.data")
    proc_mod = importlib.import_module("xkep_cae.contact.solver.process")
    nd_mod = importlib.import_module("xkep_cae.contact.solver._newton_dynamic")
    from xkep_cae.elements._beam_assembler import ULCRBeamAssembler

    m = R["tw"]._make_twisted_wire_mesh(n_wires, d, pitch, 0.0, n_el, n_pitches=1, gap=0.0)
    X, conn = m.node_coords, m.connectivity
    sec = _section(R, d)
    asm = ULCRBeamAssembler(X, conn, sec["E"], sec["G"], sec["A"], sec["Iy"], sec["Iz"], sec["J"], sec["kappa_y"],
                            sec["kappa_z"])
    M = asm.assemble_mass(rho, lumped=True)
    ndof = 6 * len(X)
    layer = np.zeros(len(conn), dtype=np.int64)
    for k, (e0, e1) in enumerate(m.strand_elem_ranges):
        layer[e0:e1] = m.strand_infos[k].layer
    fixed, pd, pv = [], [], []
    L = m.length
    for n0, n1 in m.strand_node_ranges:
        fixed += list(range(6 * n0, 6 * n0 + 6))
        ne = n1 - 1
        x, y = X[ne, 0], X[ne, 1]
        if twist != 0.0:
            c, s = math.cos(twist), math.sin(twist)
            vals = [x * (c - 1.0) - y * s, x * s + y * (c - 1.0), 0.0, 0.0, 0.0, twist]
        else:
            phi = kappa * L
            dyc, dzc = -(1.0 - math.cos(phi)) / kappa, math.sin(phi) / kappa - L
            vals = [0.0, dyc + y * (math.cos(phi) - 1.0), dzc + y * math.sin(phi), phi, 0.0, 0.0]
        pd += [6 * ne + k for k in range(6)]
        pv += vals
    k_pen = kpen_scale * sec["E"] * sec["A"] / float(np.mean(np.linalg.norm(X[conn[:, 1]] - X[conn[:, 0]], axis=1)))
    cfg = R["cp"]._ContactConfigInput(k_t_ratio=0.5, mu=mu, g_on=0.0, g_off=1e-6, exclude_same_layer=True,
                                      elem_layer_map={int(e): int(l) for e, l in enumerate(layer)},
                                      adjust_initial_penetration=False, smoothing_delta=smoothing_delta,
                                      beam_E=sec["E"], beam_I=sec["Iy"], beam_A=sec["A"],
                                      dt_max_fraction=dt_max_fraction)
    setup = data.ContactSetupData(manager=R["cp"]._ContactManagerInput(config=cfg), k_pen=k_pen, mu=mu)
    inp = data.ContactFrictionInputData(
        mesh=data.MeshData(node_coords=X, connectivity=conn, radii=np.full(len(conn), d / 2.0), n_strands=n_wires),
        boundary=data.BoundaryData(fixed_dofs=np.array(fixed), prescribed_dofs=np.array(pd),
                                   prescribed_values=np.array(pv), f_ext_total=np.zeros(ndof)),
        contact=setup,
        callbacks=data.AssembleCallbacks(assemble_tangent=asm.assemble_tangent,
                                         assemble_internal_force=asm.assemble_internal_force, ul_assembler=None),
        mass_matrix=M, dt_physical=t_total, rho_inf=rho_inf)
    calls = []
    cls = nd_mod.NewtonDynamicProcess
    orig = cls.process

    def recording(self, step_input):  # records every Newton call; changes nothing
        out = orig(self, step_input)
        calls.append((step_input.load_frac, out.converged, out.n_attempts, out.n_active,
                      list(out.diagnostics.res_history)))
        return out

    cls.process = recording
    try:
        res = proc_mod.ContactFrictionProcess().process(inp)
    finally:
        cls.process = orig
    out = {"X": X, "conn": conn, "radius": d / 2.0, "elem_layer": layer, "mass": M.diagonal(),
           "fixed": np.array(fixed), "prescribed_dofs": np.array(pd), "prescribed_values": np.array(pv),
           "k_pen": k_pen, "mu": mu, "k_t_ratio": 0.5, "smoothing_delta": smoothing_delta, "t_total": t_total,
           "rho_inf": rho_inf, "dt_max_fraction": dt_max_fraction, "converged": res.converged,
           "n_increments": res.n_increments, "n_cutbacks": res.n_cutbacks, "u_final": res.u,
           "load_history": np.array(res.load_history), "u_history": np.array(res.displacement_history),
           "inc_attempts": np.array([g.n_attempts for g in res.increment_diagnostics]),
           "inc_active": np.array([g.n_active for g in res.increment_diagnostics]),
           "call_frac": np.array([c[0] for c in calls]), "call_converged": np.array([c[1] for c in calls]),
           "call_attempts": np.array([c[2] for c in calls]), "call_active": np.array([c[3] for c in calls]),
           "call_res_ptr": np.cumsum([0] + [len(c[4]) for c in calls]),
           "call_res": np.concatenate([c[4] for c in calls]) if calls else np.zeros(0)}
    for k, v in sec.items():
        out[k] = v
    np.savez_compressed(HERE / f"{name}.npz", **out)


def protocols_case(R, name):
    """Method names and parameter names, in order, of the Strategy Protocols
    (``xkep_cae/core/strategies/protocols.py:17-256``), as JSON."""
    import importlib
    import inspect
    import json

    mod = importlib.import_module("xkep_cae.core.strategies.protocols")
    out = {}
    for proto in ("ContactForceStrategy", "FrictionStrategy", "ContactGeometryStrategy", "PenaltyStrategy",
                  "TimeIntegrationStrategy"):
        p = getattr(mod, proto)
        out[proto] = {n: [q for q in inspect.signature(v).parameters if q != "self"]
                      for n, v in vars(p).items() if callable(v) and not n.startswith("_")}
    (HERE / f"{name}.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")


CASES = {
    "protocols": lambda R: protocols_case(R, "protocols"),
    "solve7_bend": lambda R: solve_case(R, "solve7_bend", kappa=1.0 / (50.0 * 6.0)),
    "strand7":lambda R: strand_case(R, "strand7", n_wires=7, d=2.0, pitch=40.0, n_pitches=1, n_el=16,
                                     gap_frac=-0.005, seed=0, mu=0.1),
    "strand7_nogap": lambda R: strand_case(R, "strand7_nogap", n_wires=7, d=2.0, pitch=40.0, n_pitches=1, n_el=16,
                                           gap_frac=0.0, seed=0, mu=0.1, n_iter=1, n_incr=1),
    "strand19_slip": lambda R: strand_case(R, "strand19_slip", n_wires=19, d=1.0, pitch=20.0, n_pitches=1, n_el=16,
                                           gap_frac=-0.01, seed=5, mu=0.3, k_t_ratio=2.0, smoothing_delta=400.0,
                                           step_frac=2e-3, n_iter=2, n_incr=2),
    "narrowphase": lambda R: narrowphase_case(R, "narrowphase"),
    "beam_elements": lambda R: beam_case(R, "beam_elements"),
    "meshes": lambda R: mesh_case(R, "meshes"),
    "laws": lambda R: laws_case(R, "laws"),
    "genalpha": lambda R: genalpha_case(R, "genalpha"),
    "gauss_points": lambda R: gauss_case(R, "gauss_points"),
    "coating7": lambda R: coating_case(R, "coating7"),
}


def main():
    """make_golden.py /path/to/xkep-cae [case ...]  (all cases when none are named)"""
    root = sys.argv[1] if len(sys.argv) > 1 else None
    if root is None:
        raise SystemExit("usage: make_golden.py /path/to/xkep-cae [case ...]")
    R = _import_reference(root)
    for name in (sys.argv[2:] or list(CASES)):
        CASES[name](R)


if __name__ == "__main__":
    main()
