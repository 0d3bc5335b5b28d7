"""Oracle: corotational Timoshenko 3-D beam internal force and tangent (NumPy).

Restates the batched path the reference solver uses,
``_assemble_cr_beam3d_batch_impl`` (``xkep_cae/elements/_beam_assembly.py:211-325``)
with its helpers (``xkep_cae/elements/_beam_cr.py:672-998``), and the COO->CSR
assembly of ``assemble_cr_beam3d`` (``_beam_assembly.py:26-152``).
TEST INFRASTRUCTURE ONLY.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp


@dataclass(frozen=True)
class Section:
    """Material and section constants of a beam (``ULCRBeamAssembler.__init__``)."""

    E: float
    G: float
    A: float
    Iy: float
    Iz: float
    J: float
    kappa_y: float
    kappa_z: float
    scf: float | None = None


def _skew(v):
    """Stacked cross-product matrices [v]x, shape (n,3,3) (``_beam_cr.py:672``)."""
    S = np.zeros(v.shape[:-1] + (3, 3))
    S[..., 0, 1] = -v[..., 2]
    S[..., 0, 2] = v[..., 1]
    S[..., 1, 0] = v[..., 2]
    S[..., 1, 2] = -v[..., 0]
    S[..., 2, 0] = -v[..., 1]
    S[..., 2, 1] = v[..., 0]
    return S


def _mm(A, B):
    return np.einsum("nij,njk->nik", A, B)


def _mv(A, x):
    return np.einsum("nij,nj->ni", A, x)


def local_axes(ex, v_ref=None):
    """Rows (e_x, e_y, e_z) of the element frame (``_beam_cr.py:831-853``).

    Without ``v_ref`` the helper axis is the unit vector of the smallest
    |component| of e_x (first index on ties).
    """
    n = ex.shape[0]
    if v_ref is None:
        vr = np.zeros((n, 3))
        vr[np.arange(n), np.argmin(np.abs(ex), axis=1)] = 1.0
    else:
        vr = np.broadcast_to(np.asarray(v_ref, dtype=float), (n, 3))
    ez = np.cross(ex, vr)
    ez = ez / np.maximum(np.linalg.norm(ez, axis=1, keepdims=True), 1e-10)
    ey = np.cross(ez, ex)
    return np.stack([ex, ey, ez], axis=1)


def rotvec_to_rotmat(th):
    """Exponential map through the unit quaternion (``_beam_cr.py:685-726``)."""
    ang = np.linalg.norm(th, axis=1)
    small = ang < 1e-12
    half = ang / 2.0
    hsq = half * half
    safe = np.where(small, 1.0, ang)
    sinc = np.where(small, 0.5 - hsq / 48.0, np.sin(half) / safe)
    w = np.where(small, 1.0 - hsq / 2.0, np.cos(half))
    x, y, z = (sinc[:, None] * th).T
    R = np.empty((th.shape[0], 3, 3))
    R[:, 0, 0] = 1.0 - 2.0 * (y * y + z * z)
    R[:, 0, 1] = 2.0 * (x * y - w * z)
    R[:, 0, 2] = 2.0 * (x * z + w * y)
    R[:, 1, 0] = 2.0 * (x * y + w * z)
    R[:, 1, 1] = 1.0 - 2.0 * (x * x + z * z)
    R[:, 1, 2] = 2.0 * (y * z - w * x)
    R[:, 2, 0] = 2.0 * (x * z - w * y)
    R[:, 2, 1] = 2.0 * (y * z + w * x)
    R[:, 2, 2] = 1.0 - 2.0 * (x * x + y * y)
    return R


def rotmat_to_rotvec(R):
    """Logarithm map: Shepperd quaternion with the argmax branch (``_beam_cr.py:729-787``)."""
    n = R.shape[0]
    tr = R[:, 0, 0] + R[:, 1, 1] + R[:, 2, 2]
    branch = np.argmax(np.stack([tr, R[:, 0, 0], R[:, 1, 1], R[:, 2, 2]], axis=1), axis=1)
    q = np.empty((n, 4))
    # branch 0: w is the largest component
    m = branch == 0
    s = 2.0 * np.sqrt(tr[m] + 1.0)
    q[m] = np.stack([0.25 * s, (R[m, 2, 1] - R[m, 1, 2]) / s, (R[m, 0, 2] - R[m, 2, 0]) / s,
                     (R[m, 1, 0] - R[m, 0, 1]) / s], axis=1)
    m = branch == 1
    s = 2.0 * np.sqrt(1.0 + R[m, 0, 0] - R[m, 1, 1] - R[m, 2, 2])
    q[m] = np.stack([(R[m, 2, 1] - R[m, 1, 2]) / s, 0.25 * s, (R[m, 0, 1] + R[m, 1, 0]) / s,
                     (R[m, 0, 2] + R[m, 2, 0]) / s], axis=1)
    m = branch == 2
    s = 2.0 * np.sqrt(1.0 + R[m, 1, 1] - R[m, 0, 0] - R[m, 2, 2])
    q[m] = np.stack([(R[m, 0, 2] - R[m, 2, 0]) / s, (R[m, 0, 1] + R[m, 1, 0]) / s, 0.25 * s,
                     (R[m, 1, 2] + R[m, 2, 1]) / s], axis=1)
    m = branch == 3
    s = 2.0 * np.sqrt(1.0 + R[m, 2, 2] - R[m, 0, 0] - R[m, 1, 1])
    q[m] = np.stack([(R[m, 1, 0] - R[m, 0, 1]) / s, (R[m, 0, 2] + R[m, 2, 0]) / s,
                     (R[m, 1, 2] + R[m, 2, 1]) / s, 0.25 * s], axis=1)
    q[q[:, 0] < 0] *= -1.0
    q = q / np.maximum(np.linalg.norm(q, axis=1, keepdims=True), 1e-15)
    v = q[:, 1:4]
    sh = np.linalg.norm(v, axis=1)
    small = sh < 1e-12
    coef = np.where(small, 2.0, 2.0 * np.arctan2(sh, q[:, 0]) / np.where(small, 1.0, sh))
    return coef[:, None] * v


def rodrigues(e_from, e_to):
    """Smallest rotation taking e_from onto e_to (``_beam_cr.py:790-828``)."""
    v = np.cross(e_from, e_to)
    s = np.linalg.norm(v, axis=1)
    c = np.sum(e_from * e_to, axis=1)
    small = s < 1e-14
    V = _skew(v)
    coef = np.where(small, 0.0, (1.0 - c) / np.where(small, 1.0, s * s))
    R = np.eye(3)[None] + V + coef[:, None, None] * _mm(V, V)
    R[small & (c > 0)] = np.eye(3)
    for i in np.where(small & (c <= 0))[0]:
        a = np.abs(e_from[i])
        k = 0 if (a[0] <= a[1] and a[0] <= a[2]) else (1 if a[1] <= a[2] else 2)
        perp = np.zeros(3)
        perp[k] = 1.0
        ax = np.cross(e_from[i], perp)
        ax /= np.linalg.norm(ax)
        R[i] = 2.0 * np.outer(ax, ax) - np.eye(3)
    return R


def tangent_op(th):
    """T_s(theta) of the exponential map (``_beam_cr.py:856-881``)."""
    a = np.linalg.norm(th, axis=1)
    S = _skew(th)
    S2 = _mm(S, S)
    small = a < 1e-10
    sa = np.where(small, 1.0, a)
    c1 = np.where(small, 0.5, (1.0 - np.cos(sa)) / (sa * sa))
    c2 = np.where(small, 1.0 / 6.0, (1.0 - np.sin(sa) / sa) / (sa * sa))
    return np.eye(3)[None] + c1[:, None, None] * S + c2[:, None, None] * S2


def tangent_op_inv(th):
    """T_s(theta)^-1 (``_beam_cr.py:884-908``)."""
    a = np.linalg.norm(th, axis=1)
    S = _skew(th)
    S2 = _mm(S, S)
    small = a < 1e-10
    sa = np.where(small, 1.0, a)
    c = np.where(small, 1.0 / 12.0, 1.0 / (sa * sa) - (1.0 + np.cos(sa)) / (2.0 * sa * np.sin(sa)))
    return np.eye(3)[None] - 0.5 * S + c[:, None, None] * S2


def ke_local(sec: Section, L):
    """Local 12x12 Timoshenko stiffness per element length (``_beam_cr.py:911-998``)."""
    L = np.asarray(L, dtype=float)
    n = L.shape[0]
    phy = 12.0 * sec.E * sec.Iy / (sec.kappa_y * sec.G * sec.A * L * L)
    phz = 12.0 * sec.E * sec.Iz / (sec.kappa_z * sec.G * sec.A * L * L)
    if sec.scf is not None and sec.scf > 0.0:
        phy = phy / (1.0 + sec.scf * L * L * sec.A / (12.0 * sec.Iy))
        phz = phz / (1.0 + sec.scf * L * L * sec.A / (12.0 * sec.Iz))
    K = np.zeros((n, 12, 12))
    ea = sec.E * sec.A / L
    gj = sec.G * sec.J / L
    for (i, j), v in {(0, 0): ea, (0, 6): -ea, (6, 0): -ea, (6, 6): ea,
                      (3, 3): gj, (3, 9): -gj, (9, 3): -gj, (9, 9): gj}.items():
        K[:, i, j] = v
    # bending in the local x-y plane (w = u_y, rotation theta_z) and x-z plane
    for I, ph, sgn, (t, r1, t2, r2) in ((sec.Iz, phz, 1.0, (1, 5, 7, 11)),
                                         (sec.Iy, phy, -1.0, (2, 4, 8, 10))):
        den = 1.0 + ph
        k3 = 12.0 * sec.E * I / (L * L * L) / den
        k2 = 6.0 * sec.E * I / (L * L) / den
        k1a = (4.0 + ph) * sec.E * I / L / den
        k1b = (2.0 - ph) * sec.E * I / L / den
        vals = {
            (t, t): k3, (t, r1): sgn * k2, (t, t2): -k3, (t, r2): sgn * k2,
            (r1, r1): k1a, (r1, t2): -sgn * k2, (r1, r2): k1b,
            (t2, t2): k3, (t2, r2): -sgn * k2, (r2, r2): k1a,
        }
        for (i, j), v in vals.items():
            K[:, i, j] = v
            K[:, j, i] = v
    return K


def element_dofs(conn):
    conn = np.asarray(conn, dtype=np.int64)
    return (conn[:, :, None] * 6 + np.arange(6)[None, None, :]).reshape(-1, 12)


def element_batch(X0, conn, u, sec: Section, *, v_ref=None, stiffness=True, internal_force=True):
    """Per-element global force (n,12) and symmetric tangent (n,12,12)."""
    conn = np.asarray(conn, dtype=np.int64)
    edofs = element_dofs(conn)
    ue = u[edofs]
    xa, xb = X0[conn[:, 0]], X0[conn[:, 1]]
    dx0 = xb - xa
    L0 = np.linalg.norm(dx0, axis=1)
    ex0 = dx0 / L0[:, None]
    R0 = local_axes(ex0, v_ref)
    dxd = (xb + ue[:, 6:9]) - (xa + ue[:, 0:3])
    Ld = np.linalg.norm(dxd, axis=1)
    exd = dxd / Ld[:, None]
    Rcr = np.einsum("nij,nkj->nik", R0, rodrigues(ex0, exd))
    R0t = np.swapaxes(R0, 1, 2)
    th1 = rotmat_to_rotvec(_mm(_mm(Rcr, rotvec_to_rotmat(ue[:, 3:6])), R0t))
    th2 = rotmat_to_rotvec(_mm(_mm(Rcr, rotvec_to_rotmat(ue[:, 9:12])), R0t))
    d = np.zeros((len(conn), 12))
    d[:, 3:6] = th1
    d[:, 6] = Ld - L0
    d[:, 9:12] = th2
    Ke = ke_local(sec, L0)
    fcr = _mv(Ke, d)
    Rt = np.swapaxes(Rcr, 1, 2)
    fe = None
    if internal_force:
        fe = np.concatenate([_mv(Rt, fcr[:, 3 * b : 3 * b + 3]) for b in range(4)], axis=1)
    Kt = None
    if stiffness:
        dpsi1 = _mm(Rcr, _skew(exd)) / Ld[:, None, None]
        Ti1, Ti2 = tangent_op_inv(th1), tangent_op_inv(th2)
        B = np.zeros((len(conn), 12, 12))
        B[:, 6, 0:3] = -exd
        B[:, 6, 6:9] = exd
        for rows, Ti, Ts, cols in ((slice(3, 6), Ti1, tangent_op(ue[:, 3:6]), slice(3, 6)),
                                   (slice(9, 12), Ti2, tangent_op(ue[:, 9:12]), slice(9, 12))):
            P = _mm(Ti, dpsi1)
            B[:, rows, 0:3] = P
            B[:, rows, 6:9] = -P
            B[:, rows, cols] = _mm(_mm(Ti, Rcr), Ts)
        KB = _mm(Ke, B)
        Kt = np.empty((len(conn), 12, 12))
        for b in range(4):
            r = slice(3 * b, 3 * b + 3)
            G = _mm(_mm(Rt, _skew(fcr[:, r])), dpsi1)
            Kt[:, r, :] = _mm(Rt, KB[:, r, :])
            Kt[:, r, 0:3] += G
            Kt[:, r, 6:9] -= G
        Kt = 0.5 * (Kt + np.swapaxes(Kt, 1, 2))
    return fe, Kt


def assemble_beam(X0, conn, u, sec: Section, *, v_ref=None, stiffness=True, internal_force=True):
    """Global (K_T csr, f_int) as ``assemble_cr_beam3d`` returns them."""
    ndof = 6 * X0.shape[0]
    edofs = element_dofs(conn)
    fe, Ke = element_batch(X0, conn, u, sec, v_ref=v_ref, stiffness=stiffness,
                           internal_force=internal_force)
    f = None
    if internal_force:
        f = np.zeros(ndof)
        np.add.at(f, edofs.ravel(), fe.ravel())
    K = None
    if stiffness:
        rows = np.repeat(edofs, 12, axis=1).ravel()
        cols = np.tile(edofs, (1, 12)).ravel()
        K = sp.csr_matrix((Ke.reshape(-1), (rows, cols)), shape=(ndof, ndof))
        K.sum_duplicates()
    return K, f


def lumped_mass_diag(X0, conn, rho, sec: Section):
    """Diagonal of the lumped mass matrix (``_beam_assembler.py:148-169``)."""
    conn = np.asarray(conn, dtype=np.int64)
    L = np.linalg.norm(X0[conn[:, 1]] - X0[conn[:, 0]], axis=1)
    m = rho * sec.A * L
    mt = rho * (sec.Iy + sec.Iz) * L
    ri = m * L * L / 78.0
    d = np.stack([m / 2, m / 2, m / 2, mt / 2, ri, ri], axis=1)
    out = np.zeros(6 * X0.shape[0])
    edofs = element_dofs(conn)
    np.add.at(out, edofs[:, 0:6].ravel(), d.ravel())
    np.add.at(out, edofs[:, 6:12].ravel(), d.ravel())
    return out
