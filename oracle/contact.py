"""Oracle: broadphase, narrowphase, Huber normal force and Coulomb friction (NumPy).

TEST INFRASTRUCTURE ONLY.  Restates, over a structure-of-arrays pair table, the
reference's contact hot path:

* ``_broadphase_aabb``              ``xkep_cae/contact/_broadphase.py:13-96``
* ``DetectCandidatesProcess``       ``xkep_cae/contact/_manager_process.py:172-286``
* ``UpdateGeometryProcess``         ``_manager_process.py:327-403,475-494``
* ``_closest_point_segments_batch`` ``xkep_cae/contact/geometry/_compute.py:55-151``
* ``_build_contact_frame_batch``    ``_compute.py:154-261``
* ``HuberContactForceProcess``      ``xkep_cae/contact/contact_force/strategy.py:104-254``
* ``CoulombReturnMappingProcess``   ``xkep_cae/contact/friction/strategy.py:111-164``,
  ``friction/_assembly.py:53-342``, ``friction/law_friction.py:89-153``
* ``_build_constraint_jacobian_ptp`` ``xkep_cae/contact/geometry/strategy.py:83-132``
* ``_auto_select_n_gauss``          ``xkep_cae/contact/geometry/_compute.py:264-291``
* ``KelvinVoigtCoatingProcess``     ``xkep_cae/contact/coating/strategy.py:80-376`` and the
  coating branch of ``UpdateGeometryProcess`` (``_manager_process.py:351-360,386-396,475-494``)

Where the reference's candidate and active sets hinge on floating-point
compares, this oracle reproduces its arithmetic operation for operation:
``np.einsum('ij,ij->i')`` on 3-vectors sums the products as ``(p0+p2)+p1``
on the x86 NumPy build the reference was measured with, while
``np.linalg.norm(axis=1)`` and ``np.sum(axis=1)`` sum ``(p0+p1)+p2``.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

INACTIVE, ACTIVE, SLIDING = 0, 1, 2
TOL_PARALLEL = 1e-10


def dot_es(a, b):
    """``np.einsum('ij,ij->i', a, b)`` for 3-vectors: ``(a0 b0 + a2 b2) + a1 b1``."""
    return (a[:, 0] * b[:, 0] + a[:, 2] * b[:, 2]) + a[:, 1] * b[:, 1]


def dot_seq(a, b):
    """``np.sum(a*b, axis=1)`` / ``np.linalg.norm`` order: ``(a0 b0 + a1 b1) + a2 b2``."""
    return (a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1]) + a[:, 2] * b[:, 2]


def cross(a, b):
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], axis=1)


# --------------------------------------------------------------------------- pair table


def empty_table() -> dict:
    return new_pairs(np.zeros((0, 2), dtype=np.int64), np.zeros((0, 2), dtype=np.int64),
                     np.zeros(0), np.zeros(0))


def new_pairs(keys, conn, radii, core_radii=None) -> dict:
    """Fresh pair records for candidate keys ``(a<b)`` (``_contact_pair.py:38-81``)."""
    keys = np.asarray(keys, dtype=np.int64).reshape(-1, 2)
    conn = np.asarray(conn, dtype=np.int64)
    radii = np.asarray(radii, dtype=float)
    cr = radii if core_radii is None else np.asarray(core_radii, dtype=float)
    P = keys.shape[0]
    nodes = np.concatenate([conn[keys[:, 0]], conn[keys[:, 1]]], axis=1) if P else np.zeros((0, 4), np.int64)
    return {
        "ea": keys[:, 0].copy(), "eb": keys[:, 1].copy(), "nodes": nodes,
        "ra": radii[keys[:, 0]] if P else np.zeros(0), "rb": radii[keys[:, 1]] if P else np.zeros(0),
        "cra": cr[keys[:, 0]] if P else np.zeros(0), "crb": cr[keys[:, 1]] if P else np.zeros(0),
        "s": np.zeros(P), "t": np.zeros(P), "gap": np.zeros(P),
        "normal": np.zeros((P, 3)), "t1": np.zeros((P, 3)), "t2": np.zeros((P, 3)),
        "lambda_n": np.zeros(P), "k_pen": np.zeros(P), "k_t": np.zeros(P), "p_n": np.zeros(P),
        "z_t": np.zeros((P, 2)), "q_trial_norm": np.zeros(P), "status": np.zeros(P, np.int8),
        "stick": np.ones(P, bool), "dissipation": np.zeros(P),
    }


PER_PAIR = ("ea", "eb", "nodes", "ra", "rb", "cra", "crb", "s", "t", "gap", "normal", "t1", "t2",
            "lambda_n", "k_pen", "k_t", "p_n", "z_t", "q_trial_norm", "status", "stick", "dissipation")


def take(table: dict, idx) -> dict:
    return {k: table[k][idx] for k in PER_PAIR}


def concat(a: dict, b: dict) -> dict:
    return {k: np.concatenate([a[k], b[k]]) for k in PER_PAIR}


def copy_table(table: dict) -> dict:
    return {k: table[k].copy() for k in PER_PAIR}


# --------------------------------------------------------------------------- broadphase


def segment_aabbs(coords, conn, radii, margin=0.0):
    """Inflated closed AABBs ``min/max(x0,x1) -/+ (r + margin)`` (``_broadphase.py:44-49``)."""
    conn = np.asarray(conn, dtype=np.int64)
    x0, x1 = coords[conn[:, 0]], coords[conn[:, 1]]
    r = np.broadcast_to(np.asarray(radii, dtype=float), (conn.shape[0],))
    ex = (r + margin)[:, None]
    return np.minimum(x0, x1) - ex, np.maximum(x0, x1) + ex


def _expand_ranges(first, count):
    """Flat indices ``first[k] + r`` for ``r < count[k]``, and the owner ``k`` of each."""
    total = int(count.sum())
    owner = np.repeat(np.arange(count.size), count)
    offs = np.arange(total) - np.repeat(np.cumsum(count) - count, count)
    return owner, np.repeat(first, count) + offs


def aabb_overlap_pairs(lo, hi, chunk=1 << 22):
    """All pairs ``i<j`` whose closed AABBs overlap on every axis, sorted.

    The reference bins AABBs into a uniform hash grid and then keeps the pairs
    that overlap (``_broadphase.py:52-96``); every overlapping pair shares a
    cell, so its output is exactly this set whatever the cell size.  Here the
    cell is the largest box extent (a box covers at most two cells per axis),
    and a pair is tested only in the cell that holds the lower corner of the
    two boxes' intersection, the one cell that both boxes cover whenever they
    overlap, so that no pair is produced twice.
    """
    n = lo.shape[0]
    if n < 2:
        return np.zeros((0, 2), dtype=np.int64)
    base = lo.min(0)
    cell = float(np.max(hi - lo))
    if not cell > 0.0:
        cell = 1.0
    c0 = np.floor((lo - base) / cell).astype(np.int64)
    c1 = np.floor((hi - base) / cell).astype(np.int64)
    dims = c1.max(0) + 1
    span = c1 - c0 + 1
    per = span.prod(1)
    box, k = _expand_ranges(np.zeros(n, dtype=np.int64), per)
    sx, sy = span[box, 0], span[box, 1]
    cx = c0[box, 0] + k % sx
    cy = c0[box, 1] + (k // sx) % sy
    cz = c0[box, 2] + k // (sx * sy)
    key = (cz * dims[1] + cy) * dims[0] + cx
    order = np.lexsort((box, key))
    key, box = key[order], box[order]
    gstart = np.flatnonzero(np.r_[True, key[1:] != key[:-1]])
    gsize = np.diff(np.r_[gstart, key.size])
    pos = np.arange(key.size) - np.repeat(gstart, gsize)
    partners = np.repeat(gsize, gsize) - 1 - pos  # later entries of the same cell
    out = []
    lo_e = np.cumsum(partners) - partners
    e = 0
    while e < key.size:  # expand in slices of about ``chunk`` pairs
        stop = int(np.searchsorted(lo_e, lo_e[e] + chunk, side="right"))
        stop = max(stop, e + 1)
        owner, other = _expand_ranges(np.arange(e, stop) + 1, partners[e:stop])
        owner = owner + e
        a, b = box[owner], box[other]
        ok = np.all(lo[a] <= hi[b], axis=1) & np.all(lo[b] <= hi[a], axis=1)
        a, b, kk = a[ok], b[ok], key[owner[ok]]
        home = np.floor((np.maximum(lo[a], lo[b]) - base) / cell).astype(np.int64)
        hk = (home[:, 2] * dims[1] + home[:, 1]) * dims[0] + home[:, 0]
        keep = hk == kk
        a, b = a[keep], b[keep]
        out.append(np.stack([np.minimum(a, b), np.maximum(a, b)], axis=1))
        e = stop
    pairs = np.concatenate(out) if out else np.zeros((0, 2), dtype=np.int64)
    if pairs.shape[0]:
        pairs = pairs[np.lexsort((pairs[:, 1], pairs[:, 0]))]
    return pairs.astype(np.int64)


def filter_candidates(raw, coords, conn, radii, *, elem_layer=None, exclude_same_layer=False,
                      midpoint_prescreening=True, prescreening_margin=0.0, exclude_shared=True):
    """Shared-node, same-layer and midpoint filters (``_manager_process.py:200-217,260-286``)."""
    conn = np.asarray(conn, dtype=np.int64)
    r = np.broadcast_to(np.asarray(radii, dtype=float), (conn.shape[0],))
    c = raw
    if c.shape[0] and exclude_shared:
        A, B = conn[c[:, 0]], conn[c[:, 1]]
        shared = ((A[:, 0] == B[:, 0]) | (A[:, 0] == B[:, 1]) | (A[:, 1] == B[:, 0]) | (A[:, 1] == B[:, 1]))
        c = c[~shared]
    if c.shape[0] and exclude_same_layer and elem_layer is not None:
        la, lb = elem_layer[c[:, 0]], elem_layer[c[:, 1]]
        c = c[~((la == lb) & (la >= 0))]
    if c.shape[0] and midpoint_prescreening:
        n0, n1 = conn[c[:, 0], 0], conn[c[:, 0], 1]
        m0, m1 = conn[c[:, 1], 0], conn[c[:, 1], 1]
        mid_a = 0.5 * (coords[n0] + coords[n1])
        mid_b = 0.5 * (coords[m0] + coords[m1])
        da, db, dm = coords[n1] - coords[n0], coords[m1] - coords[m0], mid_a - mid_b
        half_a = 0.5 * np.sqrt(dot_seq(da, da))
        half_b = 0.5 * np.sqrt(dot_seq(db, db))
        mid_dist = np.sqrt(dot_seq(dm, dm))
        ra, rb = r[c[:, 0]], r[c[:, 1]]
        min_possible = np.maximum(0.0, mid_dist - half_a - half_b)
        extra = prescreening_margin
        if extra <= 0.0:
            extra = float(np.mean(ra + rb)) * 0.5
        c = c[min_possible <= ra + rb + extra]
    return c


def merge_candidates(table: dict, cands, conn, radii, core_radii=None) -> dict:
    """Pair-list update of ``DetectCandidatesProcess`` (``_manager_process.py:219-250``).

    Existing pairs that are not candidates turn INACTIVE and keep the rest of
    their state; new candidates get a fresh state.  The table is kept sorted
    by ``(elem_a, elem_b)``.
    """
    cands = np.asarray(cands, dtype=np.int64).reshape(-1, 2)
    old_key = table["ea"].astype(np.int64) * (1 << 32) + table["eb"]
    new_key = cands[:, 0] * (1 << 32) + cands[:, 1]
    if old_key.size == 0:  # first detection: the fresh records, sorted by key
        fresh = new_pairs(cands, conn, radii, core_radii)
        return fresh if np.all(new_key[1:] >= new_key[:-1]) else take(fresh, np.argsort(new_key, kind="stable"))
    t = copy_table(table)
    in_new = np.isin(old_key, new_key)
    t["status"][~in_new] = INACTIVE
    fresh = new_pairs(cands[~np.isin(new_key, old_key)], conn, radii, core_radii)
    merged = concat(t, fresh)
    key = merged["ea"].astype(np.int64) * (1 << 32) + merged["eb"]
    return take(merged, np.argsort(key, kind="stable"))


# --------------------------------------------------------------------------- narrowphase


def closest_point(xA0, xA1, xB0, xB1):
    """Clamped segment-segment closest point (``_compute.py:55-151``), reference op order."""
    dA, dB, w0 = xA1 - xA0, xB1 - xB0, xA0 - xB0
    a, b, c = dot_es(dA, dA), dot_es(dA, dB), dot_es(dB, dB)
    d, e = dot_es(dA, w0), dot_es(dB, w0)
    det = a * c - b * b
    par = det < TOL_PARALLEL * np.maximum(a * c, 1e-30)
    sdet = np.where(par, 1.0, det)
    with np.errstate(invalid="ignore", divide="ignore"):
        s_unc = np.where(par, 0.0, (b * e - c * d) / sdet)
        t_unc = np.where(par, 0.0, (a * e - b * d) / sdet)
        cok, aok = c > TOL_PARALLEL, a > TOL_PARALLEL
        sc, sa = np.where(cok, c, 1.0), np.where(aok, a, 1.0)
        t_par = np.where(cok, np.clip(e / sc, 0.0, 1.0), 0.0)
        s = np.where(par, 0.0, np.clip(s_unc, 0.0, 1.0))
        t = np.where(par, t_par, np.clip(t_unc, 0.0, 1.0))
        s_cl = (s_unc < 0.0) | (s_unc > 1.0)
        t_cl = (t_unc < 0.0) | (t_unc > 1.0)
        t = np.where(s_cl & ~par, np.where(cok, np.clip((b * s + e) / sc, 0.0, 1.0), 0.0), t)
        need = t_cl & ~par
        s = np.where(need, np.where(aok, np.clip((b * t - d) / sa, 0.0, 1.0), 0.0), s)
        t = np.where(need, np.where(cok, np.clip((b * s + e) / sc, 0.0, 1.0), 0.0), t)
    diff = (xA0 + s[:, None] * dA) - (xB0 + t[:, None] * dB)
    dist = np.sqrt(dot_es(diff, diff))
    normal = diff / np.maximum(dist, 1e-30)[:, None]
    normal[dist < 1e-30] = [0.0, 0.0, 1.0]
    return s, t, dist, normal, par


def contact_frame(normals, prev_t1, prev_n):
    """Transported orthonormal contact frame (``_compute.py:154-261``)."""
    N = normals.shape[0]
    n = normals / np.maximum(np.sqrt(dot_es(normals, normals)), 1e-30)[:, None]
    t1 = np.zeros((N, 3))
    t2 = np.zeros((N, 3))
    done = np.zeros(N, bool)
    has_t1 = np.sqrt(dot_es(prev_t1, prev_t1)) > 1e-10
    has_n = np.sqrt(dot_es(prev_n, prev_n)) > 1e-10
    idx = np.where(has_t1 & has_n)[0]
    if idx.size:
        n_old = prev_n[idx] / np.maximum(np.sqrt(dot_es(prev_n[idx], prev_n[idx])), 1e-30)[:, None]
        n_new, t1_old = n[idx], prev_t1[idx]
        v = cross(n_old, n_new)
        sv = np.sqrt(dot_es(v, v))
        cv = dot_es(n_old, n_new)
        tr = t1_old.copy()
        big = sv >= 1e-12
        if big.any():
            vb = v[big]
            vxt = cross(vb, t1_old[big])
            vvxt = cross(vb, vxt)
            f = (1.0 - cv[big]) / (sv[big] * sv[big])
            tr[big] = t1_old[big] + vxt + f[:, None] * vvxt
        raw = tr - dot_es(tr, n_new)[:, None] * n_new
        nr = np.sqrt(dot_es(raw, raw))
        ok = nr > 1e-10
        vi = idx[ok]
        t1[vi] = raw[ok] / nr[ok, None]
        t2[vi] = cross(n[vi], t1[vi])
        done[vi] = True
    idx = np.where(has_t1 & ~done)[0]
    if idx.size:
        raw = prev_t1[idx] - dot_es(prev_t1[idx], n[idx])[:, None] * n[idx]
        nr = np.sqrt(dot_es(raw, raw))
        ok = nr > 1e-10
        vi = idx[ok]
        t1[vi] = raw[ok] / nr[ok, None]
        t2[vi] = cross(n[vi], t1[vi])
        done[vi] = True
    idx = np.where(~done)[0]
    if idx.size:
        ni = n[idx]
        ref = np.zeros_like(ni)
        ref[np.arange(idx.size), np.argmin(np.abs(ni), axis=1)] = 1.0
        raw = ref - dot_es(ref, ni)[:, None] * ni
        nr = np.sqrt(dot_es(raw, raw))
        t1[idx] = raw / np.maximum(nr, 1e-30)[:, None]
        t2[idx] = cross(n[idx], t1[idx])
    return n, t1, t2


def update_geometry(table: dict, coords, *, freeze_active_set=False, g_on=0.0, g_off=1e-6,
                    allow_deactivation=True) -> dict:
    """Narrowphase over every pair, then active-set hysteresis unless frozen."""
    t = copy_table(table)
    if t["ea"].shape[0] == 0:
        return t
    nd = t["nodes"]
    s, tt, dist, normal, _ = closest_point(coords[nd[:, 0]], coords[nd[:, 1]], coords[nd[:, 2]], coords[nd[:, 3]])
    gap = dist - (t["ra"] + t["rb"])
    n, t1, t2 = contact_frame(normal, t["t1"], t["normal"])
    t.update(s=s, t=tt, gap=gap, normal=n, t1=t1, t2=t2)
    if not freeze_active_set:
        st = t["status"]
        on = (st == INACTIVE) & (gap <= g_on)
        off = (st != INACTIVE) & allow_deactivation & (gap >= g_off)
        st[on] = ACTIVE
        st[off] = INACTIVE
    return t


def deformed_coords(X_ref, u):
    return X_ref + u.reshape(-1, 6)[:, 0:3]


# --------------------------------------------------------------------------- forces


def shape_coeffs(s, t):
    return np.stack([1.0 - s, s, -(1.0 - t), -t], axis=1)


def trans_dofs(nodes):
    return (nodes[:, :, None] * 6 + np.arange(3)[None, None, :]).reshape(-1, 12)


def huber(x, delta):
    if delta <= 0.0:
        return np.maximum(0.0, x)
    return np.where(x < -delta, 0.0, np.where(x > delta, x, (x + delta) ** 2 / (4.0 * delta)))


def huber_deriv(x, delta):
    if delta <= 0.0:
        return np.where(x > 0.0, 1.0, 0.0)
    return np.where(x < -delta, 0.0, np.where(x > delta, 1.0, (x + delta) / (2.0 * delta)))


def huber_delta(k_pen, smoothing_delta):
    return k_pen / smoothing_delta if smoothing_delta > 0.0 else 0.0


def softplus_normal_law(gaps, k_pen: float, lambdas, delta: float = 1e-4):
    """Smooth (softplus) normal law, ``_evaluate_smooth_normal_force_vectorized``
    (``contact/penalty/law_normal.py:129-149``): p = k softplus(x, delta),
    dp/dg = -k sigmoid(x / delta), x = -g + lambda / k, |x / delta| clipped at 30."""
    gaps = np.asarray(gaps, dtype=float)
    lambdas = np.asarray(lambdas, dtype=float)
    x = -gaps + lambdas / k_pen if k_pen > 0.0 else -gaps
    z = x / delta
    ez = np.exp(np.clip(z, -30.0, 30.0))
    sp = np.where(z > 30.0, x, np.where(z < -30.0, 0.0, delta * np.log1p(ez)))
    sig = np.where(z > 30.0, 1.0, np.where(z < -30.0, 0.0, ez / (1.0 + ez)))
    return k_pen * sp, -k_pen * sig


def huber_evaluate(table: dict, ndof: int, k_pen: float, smoothing_delta: float = 0.0):
    """Normal force; writes ``p_n`` of every non-INACTIVE pair (``strategy.py:126-170``)."""
    t = copy_table(table)
    act = t["status"] != INACTIVE
    dh = huber_delta(k_pen, smoothing_delta)
    pn = huber(k_pen * (-t["gap"]), dh)
    t["p_n"] = np.where(act, pn, t["p_n"])
    resid = np.where(t["p_n"][act] > 0.0, k_pen * t["gap"][act], 0.0)
    use = act & (t["p_n"] > 1e-30)
    f = np.zeros(ndof)
    if use.any():
        c = shape_coeffs(t["s"][use], t["t"][use])
        g = c[:, :, None] * t["normal"][use][:, None, :]
        np.add.at(f, trans_dofs(t["nodes"][use]).ravel(), (t["p_n"][use][:, None, None] * g).ravel())
    return t, f, resid


def friction_evaluate(table: dict, u, u_ref, ndof: int, k_pen: float, k_t_ratio: float, mu_eff: float):
    """Coulomb return mapping over every pair with ``p_n > 0`` (``_assembly.py:260-342``).

    Returns the updated table, the friction force, the residual and the per-pair
    friction data ``(mask, q, D_t)`` the tangent needs.  Like the reference it
    reads ``p_n`` whatever the pair's status and stores ``z_t <- q`` every call.
    """
    t = copy_table(table)
    P = t["ea"].shape[0]
    use = (t["p_n"] > 0.0) & (mu_eff > 0.0)
    init = use & (t["k_pen"] <= 0.0)
    t["k_pen"] = np.where(init, k_pen, t["k_pen"])
    t["k_t"] = np.where(init, k_pen * k_t_ratio, t["k_t"])
    du = (u - (np.zeros_like(u) if u_ref is None else u_ref)).reshape(-1, 6)[:, 0:3]
    s, tt = t["s"][:, None], t["t"][:, None]
    nd = t["nodes"]
    du_rel = ((1.0 - tt) * du[nd[:, 2]] + tt * du[nd[:, 3]]) - ((1.0 - s) * du[nd[:, 0]] + s * du[nd[:, 1]])
    dut = np.stack([np.sum(du_rel * t["t1"], axis=1), np.sum(du_rel * t["t2"], axis=1)], axis=1)
    q_tr = t["z_t"] + t["k_t"][:, None] * dut
    qn = np.sqrt(q_tr[:, 0] ** 2 + q_tr[:, 1] ** 2)
    fy = mu_eff * t["p_n"]
    stick = qn <= fy
    with np.errstate(invalid="ignore", divide="ignore"):
        q = np.where(stick[:, None], q_tr, fy[:, None] * q_tr / np.where(qn > 0, qn, 1.0)[:, None])
    diss = q[:, 0] * dut[:, 0] + q[:, 1] * dut[:, 1]
    t["z_t"] = np.where(use[:, None], q, t["z_t"])
    t["stick"] = np.where(use, stick, t["stick"])
    t["q_trial_norm"] = np.where(use, qn, t["q_trial_norm"])
    t["dissipation"] = np.where(use, diss, t["dissipation"])
    t["status"] = np.where(use, np.where(stick, ACTIVE, SLIDING), t["status"]).astype(np.int8)
    qnorm = np.sqrt(q[:, 0] ** 2 + q[:, 1] ** 2)
    fr = use & (qnorm >= 1e-30)
    resid = np.maximum(0.0, qnorm[fr] - mu_eff * t["p_n"][fr])
    # 2x2 consistent tangent (law_friction.py:126-153)
    D = np.zeros((P, 2, 2))
    eye = np.eye(2)
    kt = t["k_t"]
    D[:] = kt[:, None, None] * eye
    slip = fr & ~stick & (qn >= 1e-30) & (qnorm >= 1e-30)
    if slip.any():
        qh = q[slip] / qnorm[slip, None]
        ratio = mu_eff * t["p_n"][slip] / qn[slip]
        D[slip] = (ratio * kt[slip])[:, None, None] * (eye[None] - qh[:, :, None] * qh[:, None, :])
    f = np.zeros(ndof)
    if fr.any():
        c = shape_coeffs(t["s"][fr], t["t"][fr])
        qq = np.where(np.abs(q[fr]) < 1e-30, 0.0, q[fr])
        v = qq[:, 0:1] * t["t1"][fr] + qq[:, 1:2] * t["t2"][fr]
        np.add.at(f, trans_dofs(nd[fr]).ravel(), (c[:, :, None] * v[:, None, :]).ravel())
    return t, f, resid, {"mask": fr, "q": q, "D": D}


def _blocks_to_csr(nodes, blocks, ndof):
    """Assemble per-pair (4x4 node) x (3x3) blocks, shape (P,4,4,3,3), to CSR.

    Blocks with the same (row node, column node) are summed, then laid out as
    3x3 blocks of a block matrix whose block (2a, 2b) is the translational
    block of nodes a and b.
    """
    P = nodes.shape[0]
    if P == 0:
        return sp.csr_matrix((ndof, ndof))
    nn = ndof // 6
    nodes = np.asarray(nodes, dtype=np.int64)
    key = (nodes[:, :, None] * nn + nodes[:, None, :]).ravel()
    order = np.argsort(key, kind="stable")
    key = key[order]
    start = np.flatnonzero(np.r_[True, key[1:] != key[:-1]])
    summed = np.add.reduceat(blocks.reshape(-1, 3, 3)[order], start, axis=0)
    ukey = key[start]
    brow, bcol = 2 * (ukey // nn), 2 * (ukey % nn)
    indptr = np.searchsorted(brow, np.arange(2 * nn + 1))
    return sp.bsr_matrix((summed, bcol, indptr), shape=(ndof, ndof)).tocsr()


def huber_tangent(table: dict, ndof: int, k_pen: float, smoothing_delta: float = 0.0):
    """K_mat - K_geo of the normal force (``strategy.py:172-254``)."""
    t = table
    dh = huber_delta(k_pen, smoothing_delta)
    x = k_pen * (-t["gap"])
    hd = huber_deriv(x, dh)
    pn = t["p_n"]
    use = (t["status"] != INACTIVE) & ~((hd < 1e-30) & (pn < 1e-30))
    if not use.any():
        return sp.csr_matrix((ndof, ndof))
    n = t["normal"][use]
    dist = (t["gap"][use] + t["ra"][use]) + t["rb"][use]
    wm = hd[use] * k_pen
    wg = np.where(dist > 1e-15, pn[use] / np.where(dist > 1e-15, dist, 1.0), 0.0)
    nn = n[:, :, None] * n[:, None, :]
    Bm = wm[:, None, None] * nn - wg[:, None, None] * (np.eye(3)[None] - nn)
    c = shape_coeffs(t["s"][use], t["t"][use])
    cc = c[:, :, None] * c[:, None, :]
    blocks = cc[:, :, :, None, None] * Bm[:, None, None, :, :]
    return _blocks_to_csr(t["nodes"][use], blocks, ndof)


def friction_tangent(table: dict, fric: dict, ndof: int):
    """Material + geometric friction stiffness (``_assembly.py:108-257``)."""
    t = table
    use = fric["mask"] & (t["status"] != INACTIVE)
    if not use.any():
        return sp.csr_matrix((ndof, ndof))
    D = fric["D"][use]
    q = fric["q"][use]
    n, t1, t2 = t["normal"][use], t["t1"][use], t["t2"][use]
    tv = np.stack([t1, t2], axis=1)
    D = np.where(np.abs(D) < 1e-30, 0.0, D)
    Bmat = np.einsum("pab,pai,pbj->pij", D, tv, tv)
    dist = (t["gap"][use] + t["ra"][use]) + t["rb"][use]
    q1, q2 = q[:, 0], q[:, 1]
    M = -q1[:, None, None] * n[:, :, None] * t1[:, None, :] - q2[:, None, None] * t2[:, :, None] * n[:, None, :]
    sk = np.zeros_like(M)
    sk[:, 0, 1], sk[:, 0, 2], sk[:, 1, 0] = t1[:, 2], -t1[:, 1], -t1[:, 2]
    sk[:, 1, 2], sk[:, 2, 0], sk[:, 2, 1] = t1[:, 0], t1[:, 1], -t1[:, 0]
    M = M + q2[:, None, None] * sk
    geo_ok = (dist >= 1e-15) & ~((np.abs(q1) < 1e-30) & (np.abs(q2) < 1e-30))
    inv = np.where(geo_ok, 1.0 / np.where(dist >= 1e-15, dist, 1.0), 0.0)
    Bf = Bmat + inv[:, None, None] * M
    c = shape_coeffs(t["s"][use], t["t"][use])
    cc = c[:, :, None] * c[:, None, :]
    blocks = cc[:, :, :, None, None] * Bf[:, None, None, :, :]
    return _blocks_to_csr(t["nodes"][use], blocks, ndof)


def constraint_jacobian(table: dict, ndof: int):
    """PtP constraint Jacobian rows for non-INACTIVE pairs (``geometry/strategy.py:83-132``)."""
    act = np.where(table["status"] != INACTIVE)[0]
    if act.size == 0:
        return sp.csr_matrix((0, ndof)), []
    c = shape_coeffs(table["s"][act], table["t"][act])
    vals = (c[:, :, None] * table["normal"][act][:, None, :]).reshape(-1, 12)
    rows = np.repeat(np.arange(act.size), 12)
    cols = trans_dofs(table["nodes"][act]).ravel()
    keep = np.abs(vals.ravel()) > 1e-30
    G = sp.csr_matrix((vals.ravel()[keep], (rows[keep], cols[keep])), shape=(act.size, ndof))
    return G, [int(i) for i in act]


# --------------------------------------------------------------------------- whole assembly


def detect(table, coords, conn, radii, *, margin=0.0, elem_layer=None, exclude_same_layer=False,
           midpoint_prescreening=True, prescreening_margin=0.0, core_radii=None):
    """Broadphase + filters + pair-list merge; returns (table, candidates, raw)."""
    lo, hi = segment_aabbs(coords, conn, radii, margin)
    raw = aabb_overlap_pairs(lo, hi)
    cands = filter_candidates(raw, coords, conn, radii, elem_layer=elem_layer,
                              exclude_same_layer=exclude_same_layer,
                              midpoint_prescreening=midpoint_prescreening,
                              prescreening_margin=prescreening_margin)
    return merge_candidates(table, cands, conn, radii, core_radii), cands, raw


def contact_iteration(table, X_ref, u, u_ref, ndof, *, k_pen, k_t_ratio, mu_eff, smoothing_delta=0.0):
    """One Newton iteration's contact work, in the solver's order.

    ``ContactForceAssemblyProcess`` (``_newton_steps.py:79-135``): frozen
    narrowphase, normal force, friction; then ``TangentAssemblyProcess``
    (``:289-313``): normal tangent and friction tangent.  Returns the table,
    ``f_contact = -(f_n + f_f)`` and ``K_contact = K_n - K_f``.
    """
    t = update_geometry(table, deformed_coords(X_ref, u), freeze_active_set=True)
    t, fn, _ = huber_evaluate(t, ndof, k_pen, smoothing_delta)
    t, ff, _, fr = friction_evaluate(t, u, u_ref, ndof, k_pen, k_t_ratio, mu_eff)
    Kn = huber_tangent(t, ndof, k_pen, smoothing_delta)
    Kf = friction_tangent(t, fr, ndof)
    return t, -(fn + ff), (Kn - Kf).tocsr(), {"f_n": fn, "f_f": ff, "K_n": Kn, "K_f": Kf, "fric": fr}


def auto_n_gauss(dA, dB, default: int = 3) -> np.ndarray:
    """Gauss-point count per segment pair (``_auto_select_n_gauss``, ``geometry/_compute.py:264-291``).

    Row by row with the reference's own NumPy calls (``np.linalg.norm`` of a
    3-vector, ``dA @ dB``): |cos| < 0.866 -> 2, < 0.985 -> 3, else 5; ``default``
    when a segment has zero length.
    """
    dA = np.asarray(dA, dtype=float).reshape(-1, 3)
    dB = np.asarray(dB, dtype=float).reshape(-1, 3)
    out = np.empty(dA.shape[0], dtype=np.int64)
    for i in range(dA.shape[0]):
        len_a = float(np.linalg.norm(dA[i]))
        len_b = float(np.linalg.norm(dB[i]))
        if len_a < 1e-30 or len_b < 1e-30:
            out[i] = default
            continue
        c = abs(float(dA[i] @ dB[i] / (len_a * len_b)))
        out[i] = 2 if c < 0.866 else (3 if c < 0.985 else 5)
    return out


# --------------------------------------------------------------------------- coating


def coating_geometry(table: dict, coords, *, freeze_active_set=False, g_on=0.0, g_off=1e-6,
                     allow_deactivation=True):
    """Geometry with a coating (``_manager_process.py:351-360,386-396,475-494``).

    The gap is taken between the cores, ``dist - (core_a + core_b)``; the
    coating compression is ``max(0, coat_total - gap)`` with ``coat_total =
    (r_a - core_a) + (r_b - core_b)``; a compressed coating activates a pair
    and keeps it active.  Returns the updated table and the compressions.
    """
    t = copy_table(table)
    if t["ea"].shape[0] == 0:
        return t, np.zeros(0)
    nd = t["nodes"]
    s, tt, dist, normal, _ = closest_point(coords[nd[:, 0]], coords[nd[:, 1]], coords[nd[:, 2]], coords[nd[:, 3]])
    gap = dist - (t["cra"] + t["crb"])
    coat_total = (t["ra"] - t["cra"]) + (t["rb"] - t["crb"])
    cc = np.maximum(0.0, coat_total - gap)
    n, t1, t2 = contact_frame(normal, t["t1"], t["normal"])
    t.update(s=s, t=tt, gap=gap, normal=n, t1=t1, t2=t2)
    if not freeze_active_set:
        st = t["status"]
        coat = cc > 0.0
        on = (st == INACTIVE) & ((gap <= g_on) | coat)
        off = (st != INACTIVE) & allow_deactivation & (gap >= g_off) & ~coat
        st[on] = ACTIVE
        st[off] = INACTIVE
    return t, cc


def _assemble_nodal(table, use, v, ndof):
    f = np.zeros(ndof)
    if use.any():
        c = shape_coeffs(table["s"][use], table["t"][use])
        np.add.at(f, trans_dofs(table["nodes"][use]).ravel(), (c[:, :, None] * v[use][:, None, :]).ravel())
    return f


def coating_forces(table: dict, cc, cc_prev, ndof: int, k: float, c: float, dt: float):
    """Elastic + viscous coating force (``coating/strategy.py:97-143``): f_n = k cc + c (cc - cc_prev) / dt
    (the dashpot when c > 0 and dt > 0), on node k of a pair c_k (-f_n n)."""
    f_n = k * cc
    if c > 0.0 and dt > 0.0:
        f_n = f_n + c * ((cc - cc_prev) / dt)
    use = ~((cc <= 0.0) & (cc_prev <= 0.0)) & ~(np.abs(f_n) < 1e-30)
    return _assemble_nodal(table, use, -f_n[:, None] * table["normal"], ndof)


def coating_stiffness(table: dict, cc, ndof: int, k: float, c: float, dt: float):
    """Coating stiffness (``coating/strategy.py:145-196``): blocks c_k c_l (k + c/dt) n n^T where cc > 1e-15."""
    k_eff = k + c / dt if (c > 0.0 and dt > 0.0) else k
    use = cc > 1e-15
    if not use.any():
        return sp.csr_matrix((ndof, ndof))
    n = table["normal"][use]
    B = k_eff * n[:, :, None] * n[:, None, :]
    co = shape_coeffs(table["s"][use], table["t"][use])
    blocks = (co[:, :, None] * co[:, None, :])[:, :, :, None, None] * B[:, None, None, :, :]
    return _blocks_to_csr(table["nodes"][use], blocks, ndof)


def coating_friction(table: dict, cc, state: dict, u, u_ref, ndof: int, k: float, kt_ratio: float, mu: float):
    """Coating friction (``coating/strategy.py:198-288``): return mapping on the coating surface with
    p_n = k cc and k_t = k kt_ratio; the history of uncompressed pairs is reset.  Returns the force and
    the new state (z_t, stick, q_trial_norm, dissipation)."""
    P = table["ea"].shape[0]
    new = {key: np.array(v, copy=True) for key, v in state.items()}
    if mu <= 0.0:
        return np.zeros(ndof), new
    k_t = k * kt_ratio
    du = (u - u_ref).reshape(-1, 6)[:, 0:3]
    s, tt, nd = table["s"][:, None], table["t"][:, None], table["nodes"]
    du_rel = ((1.0 - tt) * du[nd[:, 2]] + tt * du[nd[:, 3]]) - ((1.0 - s) * du[nd[:, 0]] + s * du[nd[:, 1]])
    dut = np.stack([np.sum(du_rel * table["t1"], axis=1), np.sum(du_rel * table["t2"], axis=1)], axis=1)
    comp = cc > 0.0
    p_n = k * cc
    q_tr = state["z_t"] + k_t * dut
    qn = np.sqrt(q_tr[:, 0] ** 2 + q_tr[:, 1] ** 2)
    fy = mu * p_n
    stick = qn <= fy
    with np.errstate(invalid="ignore", divide="ignore"):
        q = np.where(stick[:, None], q_tr, fy[:, None] * q_tr / np.where(qn > 0, qn, 1.0)[:, None])
    diss = q[:, 0] * dut[:, 0] + q[:, 1] * dut[:, 1]
    new["z_t"] = np.where(comp[:, None], q, 0.0)
    new["stick"] = np.where(comp, stick, True)
    new["q_trial_norm"] = np.where(comp, qn, 0.0)
    new["dissipation"] = np.where(comp, diss, 0.0)
    v = -(new["z_t"][:, 0:1] * table["t1"] + new["z_t"][:, 1:2] * table["t2"])
    return _assemble_nodal(table, comp, v, ndof), new


def coating_friction_stiffness(table: dict, cc, state: dict, ndof: int, k: float, kt_ratio: float, mu: float):
    """Coating friction stiffness (``coating/strategy.py:290-370``): blocks c_k c_l T D T^T, D from
    ``_tangent_2x2_core`` (``friction/law_friction.py:126-153``) on the coating friction state."""
    use = (cc > 0.0) & (mu > 0.0)
    if not use.any():
        return sp.csr_matrix((ndof, ndof))
    k_t = k * kt_ratio
    p_n = k * cc[use]
    z = state["z_t"][use]
    qtn = state["q_trial_norm"][use]
    zn = np.sqrt(z[:, 0] ** 2 + z[:, 1] ** 2)
    slip = ~state["stick"][use] & (zn >= 1e-30) & (qtn >= 1e-30)
    D = np.broadcast_to(k_t * np.eye(2), (z.shape[0], 2, 2)).copy()
    if slip.any():
        h = z[slip] / zn[slip, None]
        ratio = mu * p_n[slip] / qtn[slip]
        D[slip] = (ratio * k_t)[:, None, None] * (np.eye(2)[None] - h[:, :, None] * h[:, None, :])
    tv = np.stack([table["t1"][use], table["t2"][use]], axis=1)
    B = np.einsum("pab,pai,pbj->pij", D, tv, tv)
    co = shape_coeffs(table["s"][use], table["t"][use])
    blocks = (co[:, :, None] * co[:, None, :])[:, :, :, None, None] * B[:, None, None, :, :]
    return _blocks_to_csr(table["nodes"][use], blocks, ndof)
