"""The algebra of the float beam kernel, restated in NumPy (CPU): the element tangent assembled from six
symmetrised 3x3 blocks equals the oracle's symmetrised element tangent, and the element forces its global
block forces, at large rotations.

The float kernel (``k_beam32e``) uses that rows 6..8 of the local stiffness are the negatives of rows 0..2
(so the unsymmetrised block rows are [G0 H0 -G0 J0; G1 H1 -G1 J1; -G0 -H0 G0 -J0; G3 H3 -G3 J3]), forms
each G/H/J as outer products of the rows of R_cr with scaled rows of P_s = T^-1(t_s) R_cr [e_x]x / L and
Q_s = T^-1(t_s) R_cr T(theta_node), and writes the geometric term as (e_x g^T - (g . e_x) I) / L with
g = R_cr^T f (``_assemble_cr_beam3d_batch_impl``, ``elements/_beam_assembly.py:211-325``).
"""

from __future__ import annotations

import numpy as np

from oracle import beam as ob


def _six_block_tangent(X0, conn, u, sec):
    ue = u[ob.element_dofs(conn)]
    xa, xb = X0[conn[:, 0]], X0[conn[:, 1]]
    dx0 = xb - xa
    L0 = np.linalg.norm(dx0, axis=1)
    R0 = ob.local_axes(dx0 / L0[:, None], None)
    dxd = (xb + ue[:, 6:9]) - (xa + ue[:, 0:3])
    Ld = np.linalg.norm(dxd, axis=1)
    ex = dxd / Ld[:, None]
    Rcr = np.einsum("nij,nkj->nik", R0, ob.rodrigues(dx0 / L0[:, None], ex))
    R0t = np.swapaxes(R0, 1, 2)
    t1 = ob.rotmat_to_rotvec(ob._mm(ob._mm(Rcr, ob.rotvec_to_rotmat(ue[:, 3:6])), R0t))
    t2 = ob.rotmat_to_rotvec(ob._mm(ob._mm(Rcr, ob.rotvec_to_rotmat(ue[:, 9:12])), R0t))
    Ke = ob.ke_local(sec, L0)
    ea, gj = Ke[:, 0, 0], Ke[:, 3, 3]
    k2z, k1az, k1bz = Ke[:, 1, 5], Ke[:, 5, 5], Ke[:, 5, 11]
    k2y, k1ay, k1by = -Ke[:, 2, 4], Ke[:, 4, 4], Ke[:, 4, 10]
    dax = Ld - L0
    f0 = np.stack([-ea * dax, k2z * (t1[:, 2] + t2[:, 2]), -k2y * (t1[:, 1] + t2[:, 1])], 1)
    f1 = np.stack([gj * (t1[:, 0] - t2[:, 0]), k1ay * t1[:, 1] + k1by * t2[:, 1], k1az * t1[:, 2] + k1bz * t2[:, 2]], 1)
    f3 = np.stack([-f1[:, 0], k1by * t1[:, 1] + k1ay * t2[:, 1], k1bz * t1[:, 2] + k1az * t2[:, 2]], 1)
    Rt = np.swapaxes(Rcr, 1, 2)
    g0, g1, g3 = ob._mv(Rt, f0), ob._mv(Rt, f1), ob._mv(Rt, f3)
    fe = np.concatenate([g0, g1, -g0, g3], 1)

    def pq(t, th):
        M = ob._mm(ob.tangent_op_inv(t), Rcr)
        return np.cross(M, ex[:, None, :]) / Ld[:, None, None], ob._mm(M, ob.tangent_op(th))

    P1, Q1 = pq(t1, ue[:, 3:6])
    P2, Q2 = pq(t2, ue[:, 9:12])
    R_0, R_1, R_2 = Rcr[:, 0], Rcr[:, 1], Rcr[:, 2]
    o = lambda a, b: a[:, :, None] * b[:, None, :]  # noqa: E731
    c = lambda x: x[:, None]  # noqa: E731
    G1 = o(R_0, c(gj) * (P1[:, 0] - P2[:, 0])) + o(R_1, c(k1ay) * P1[:, 1] + c(k1by) * P2[:, 1]) \
        + o(R_2, c(k1az) * P1[:, 2] + c(k1bz) * P2[:, 2])
    G3 = o(R_0, -c(gj) * (P1[:, 0] - P2[:, 0])) + o(R_1, c(k1by) * P1[:, 1] + c(k1ay) * P2[:, 1]) \
        + o(R_2, c(k1bz) * P1[:, 2] + c(k1az) * P2[:, 2])
    G0 = o(R_0, c(ea) * ex) + o(R_1, c(k2z) * (P1[:, 2] + P2[:, 2])) + o(R_2, -c(k2y) * (P1[:, 1] + P2[:, 1]))
    eye = np.eye(3)[None]

    def geo(g):
        return (o(ex, g) - np.einsum("ni,ni->n", g, ex)[:, None, None] * eye) / Ld[:, None, None]

    G0, G1, G3 = G0 + geo(g0), G1 + geo(g1), G3 + geo(g3)
    H0 = o(R_1, c(k2z) * Q1[:, 2]) + o(R_2, -c(k2y) * Q1[:, 1])
    J0 = o(R_1, c(k2z) * Q2[:, 2]) + o(R_2, -c(k2y) * Q2[:, 1])
    H1 = o(R_0, c(gj) * Q1[:, 0]) + o(R_1, c(k1ay) * Q1[:, 1]) + o(R_2, c(k1az) * Q1[:, 2])
    J3 = o(R_0, c(gj) * Q2[:, 0]) + o(R_1, c(k1ay) * Q2[:, 1]) + o(R_2, c(k1az) * Q2[:, 2])
    J1 = o(R_0, -c(gj) * Q2[:, 0]) + o(R_1, c(k1by) * Q2[:, 1]) + o(R_2, c(k1bz) * Q2[:, 2])
    H3 = o(R_0, -c(gj) * Q1[:, 0]) + o(R_1, c(k1by) * Q1[:, 1]) + o(R_2, c(k1bz) * Q1[:, 2])
    T = lambda x: np.swapaxes(x, 1, 2)  # noqa: E731
    S00, S01, S11 = 0.5 * (G0 + T(G0)), 0.5 * (H0 + T(G1)), 0.5 * (H1 + T(H1))
    S03, S13, S33 = 0.5 * (J0 + T(G3)), 0.5 * (J1 + T(H3)), 0.5 * (J3 + T(J3))
    # the stored blocks aa, ab, bb of the kernel, and the full 12 x 12 from them
    K = np.zeros((len(conn), 12, 12))
    blocks = {(0, 0): S00, (0, 1): S01, (1, 0): T(S01), (1, 1): S11,
              (0, 2): -S00, (0, 3): S03, (1, 2): -T(S01), (1, 3): S13,
              (2, 2): S00, (2, 3): -S03, (3, 2): -T(S03), (3, 3): S33}
    for (i, j), X in blocks.items():
        K[:, 3 * i:3 * i + 3, 3 * j:3 * j + 3] = X
        if i != j and (j, i) not in blocks:
            K[:, 3 * j:3 * j + 3, 3 * i:3 * i + 3] = T(X)
    return fe, K


def test_six_block_tangent_equals_oracle_at_large_rotations():
    rng = np.random.default_rng(1)
    n = 300
    X0 = np.zeros((2 * n, 3))
    d = rng.normal(size=(n, 3))
    X0[1::2] = d / np.linalg.norm(d, axis=1)[:, None] * rng.uniform(0.5, 2.0, (n, 1))
    conn = np.stack([np.arange(0, 2 * n, 2), np.arange(1, 2 * n, 2)], 1)
    u = np.zeros(12 * n)
    u6 = u.reshape(-1, 6)
    u6[:, :3] = 0.05 * rng.normal(size=(2 * n, 3))
    u6[:, 3:] = 0.5 * rng.normal(size=(2 * n, 3))  # rotations of about 0.9 rad
    for scf in (None, 0.3):
        sec = ob.Section(E=2e5, G=8e4, A=0.8, Iy=0.05, Iz=0.07, J=0.1, kappa_y=0.85, kappa_z=0.85, scf=scf)
        fe_ref, K_ref = ob.element_batch(X0, conn, u, sec)
        fe, K = _six_block_tangent(X0, conn, u, sec)
        assert np.max(np.abs(fe - fe_ref)) <= 1e-12 * np.max(np.abs(fe_ref))
        assert np.max(np.abs(K - K_ref)) <= 1e-12 * np.max(np.abs(K_ref))
