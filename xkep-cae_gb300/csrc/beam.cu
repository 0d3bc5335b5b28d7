// Corotational Timoshenko beam: internal force and analytic tangent per element.
//
// Mirrors _assemble_cr_beam3d_batch_impl (xkep_cae/elements/_beam_assembly.py:211-325)
// one element per thread.  The corotated frame is taken in double in both
// precision modes, in quaternion form:
//   R_cr = R0 R_rod^T,  theta_def = log(R_cr R_node R0^T) = R0 log(q_rod^* (x) q_node)
// which equals the reference's matrix Shepperd route for rotations below pi.
// Everything downstream of the frame (local stiffness, f_cr, B, K_mat, K_geo)
// runs in Prec<P>::T.
#include "xk_common.cuh"

namespace {

constexpr int BEAM_T = 128;

// ---- quaternion helpers (double) ----
XK_D void qmul(const double* a, const double* b, double* c) {
  c[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  c[1] = a[0] * b[1] + b[0] * a[1] + a[2] * b[3] - a[3] * b[2];
  c[2] = a[0] * b[2] + b[0] * a[2] + a[3] * b[1] - a[1] * b[3];
  c[3] = a[0] * b[3] + b[0] * a[3] + a[1] * b[2] - a[2] * b[1];
}

// Unit quaternion of the rotation vector th (exponential map, _beam_cr.py:685-726).
XK_D void quat_of_rotvec(const double* th, double* q) {
  double a2 = th[0] * th[0] + th[1] * th[1] + th[2] * th[2];
  double c, so;  // cos(a/2), sin(a/2)/a
  if (a2 < 0.0625) {  // a < 0.25: Taylor series, truncation < 1e-18
    double h2 = 0.25 * a2;
    c = 1.0 + h2 * (-1.0 / 2 + h2 * (1.0 / 24 + h2 * (-1.0 / 720 + h2 * (1.0 / 40320 + h2 * (-1.0 / 3628800)))));
    so = 0.5 * (1.0 + h2 * (-1.0 / 6 + h2 * (1.0 / 120 + h2 * (-1.0 / 5040 + h2 * (1.0 / 362880 + h2 * (-1.0 / 39916800))))));
  } else {
    double a = sqrt(a2), sh;
    sincos(0.5 * a, &sh, &c);
    so = sh / a;
  }
  q[0] = c;
  q[1] = so * th[0];
  q[2] = so * th[1];
  q[3] = so * th[2];
}

// Rotation vector of a unit quaternion (logarithm map, _beam_cr.py:771-787).
XK_D void rotvec_of_quat(const double* qin, double* th) {
  double w = qin[0], x = qin[1], y = qin[2], z = qin[3];
  if (w < 0.0) { w = -w; x = -x; y = -y; z = -z; }
  double s2 = x * x + y * y + z * z;
  double coef;
  if (s2 < 0.0025 * w * w) {  // |v|/w < 0.05: 2 atan(r)/(r w) by its series
    double r2 = s2 / (w * w);
    double at = 1.0 + r2 * (-1.0 / 3 + r2 * (1.0 / 5 + r2 * (-1.0 / 7 + r2 * (1.0 / 9 + r2 * (-1.0 / 11 + r2 * (1.0 / 13))))));
    coef = 2.0 * at / w;
  } else {
    double sh = sqrt(s2);
    coef = 2.0 * atan2(sh, w) / sh;
  }
  th[0] = coef * x;
  th[1] = coef * y;
  th[2] = coef * z;
}

// Quaternion of the smallest rotation taking unit e0 onto unit e1
// (_batch_rodrigues_rotation, _beam_cr.py:790-828).
XK_D void quat_between(const double* e0, const double* e1, double* q) {
  double v[3];
  v[0] = e0[1] * e1[2] - e0[2] * e1[1];
  v[1] = e0[2] * e1[0] - e0[0] * e1[2];
  v[2] = e0[0] * e1[1] - e0[1] * e1[0];
  double c = e0[0] * e1[0] + e0[1] * e1[1] + e0[2] * e1[2];
  double s2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  if (s2 < 1e-28) {
    if (c > 0.0) {
      q[0] = 1.0; q[1] = q[2] = q[3] = 0.0;
    } else {  // half turn about e0 x (unit vector of its smallest component)
      double ax[3], p[3] = {0.0, 0.0, 0.0};
      double a0 = fabs(e0[0]), a1 = fabs(e0[1]), a2 = fabs(e0[2]);
      p[(a0 <= a1 && a0 <= a2) ? 0 : (a1 <= a2 ? 1 : 2)] = 1.0;
      cross3(e0, p, ax);
      double n = sqrt(dot3(ax, ax));
      q[0] = 0.0; q[1] = ax[0] / n; q[2] = ax[1] / n; q[3] = ax[2] / n;
    }
    return;
  }
  double w = sqrt(0.5 * (1.0 + c));
  double k = 0.5 / w;
  q[0] = w; q[1] = k * v[0]; q[2] = k * v[1]; q[3] = k * v[2];
}

template <typename T>
XK_D void rotmat_of_quat(const double* q, T* R) {
  T w = (T)q[0], x = (T)q[1], y = (T)q[2], z = (T)q[3];
  R[0] = T(1) - T(2) * (y * y + z * z); R[1] = T(2) * (x * y - w * z); R[2] = T(2) * (x * z + w * y);
  R[3] = T(2) * (x * y + w * z); R[4] = T(1) - T(2) * (x * x + z * z); R[5] = T(2) * (y * z - w * x);
  R[6] = T(2) * (x * z - w * y); R[7] = T(2) * (y * z + w * x); R[8] = T(1) - T(2) * (x * x + y * y);
}

// Float versions of the exponential / logarithm maps and quaternion product for
// the mixed path (small rotation vectors by their series, as in double).
XK_D void qmulf(const float* a, const float* b, float* c) {
  c[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  c[1] = a[0] * b[1] + b[0] * a[1] + a[2] * b[3] - a[3] * b[2];
  c[2] = a[0] * b[2] + b[0] * a[2] + a[3] * b[1] - a[1] * b[3];
  c[3] = a[0] * b[3] + b[0] * a[3] + a[1] * b[2] - a[2] * b[1];
}
XK_D void quat_of_rotvecf(const float* th, float* q) {
  const float a2 = th[0] * th[0] + th[1] * th[1] + th[2] * th[2];
  float c, so;
  if (a2 < 0.0625f) {
    const float h2 = 0.25f * a2;
    c = 1.0f + h2 * (-0.5f + h2 * (1.0f / 24 + h2 * (-1.0f / 720 + h2 * (1.0f / 40320))));
    so = 0.5f * (1.0f + h2 * (-1.0f / 6 + h2 * (1.0f / 120 + h2 * (-1.0f / 5040 + h2 * (1.0f / 362880)))));
  } else {
    const float a = sqrtf(a2);
    float sh;
    sincosf(0.5f * a, &sh, &c);
    so = sh / a;
  }
  q[0] = c;
  q[1] = so * th[0];
  q[2] = so * th[1];
  q[3] = so * th[2];
}
XK_D void rotvec_of_quatf(const float* qin, float* th) {
  float w = qin[0], x = qin[1], y = qin[2], z = qin[3];
  if (w < 0.0f) { w = -w; x = -x; y = -y; z = -z; }
  const float s2 = x * x + y * y + z * z;
  float coef;
  if (s2 < 0.0025f * w * w) {
    const float r2 = s2 / (w * w);
    coef = 2.0f * (1.0f + r2 * (-1.0f / 3 + r2 * (1.0f / 5 + r2 * (-1.0f / 7 + r2 * (1.0f / 9))))) / w;
  } else {
    const float sh = sqrtf(s2);
    coef = 2.0f * atan2f(sh, w) / sh;
  }
  th[0] = coef * x;
  th[1] = coef * y;
  th[2] = coef * z;
}

// T_s(theta) = I + c1 S + c2 S^2 and T_s^{-1} = I - S/2 + c3 S^2 (_beam_cr.py:856-908),
// with series below |theta| = 0.25 so that the float path keeps its accuracy.
// The float instantiation takes the series up to |theta| = 1, where the truncated terms are
// below 1e-10 of the sums and the closed forms no longer cancel in float, and evaluates the
// closed forms with the float sincos: no double arithmetic in the mixed beam kernel.
template <typename T>
XK_D void tangent_ops(const T* th, bool inverse, T* M) {
  T a2 = th[0] * th[0] + th[1] * th[1] + th[2] * th[2];
  T c1, c2;
  constexpr bool F32 = sizeof(T) == 4;
  if (a2 < (F32 ? T(1) : T(0.0625))) {
    if (!inverse) {
      c1 = T(0.5) + a2 * (T(-1.0 / 24) + a2 * (T(1.0 / 720) + a2 * (T(-1.0 / 40320) + a2 * (T(1.0 / 3628800) + a2 * T(-1.0 / 479001600)))));
      c2 = T(1.0 / 6) + a2 * (T(-1.0 / 120) + a2 * (T(1.0 / 5040) + a2 * (T(-1.0 / 362880) + a2 * (T(1.0 / 39916800) + a2 * T(-1.0 / 6227020800.0)))));
    } else {
      c1 = T(-0.5);
      c2 = T(1.0 / 12) + a2 * (T(1.0 / 720) + a2 * (T(1.0 / 30240) + a2 * (T(1.0 / 1209600) + a2 * (T(1.0 / 47900160) + a2 * T(691.0 / 1307674368000.0)))));
    }
  } else {
    T a = my_sqrt<T>(a2);
    T s, c;
    if (F32) {
      float sf, cf;
      sincosf((float)a, &sf, &cf);
      s = (T)sf;
      c = (T)cf;
    } else {
      double sd, cd;
      sincos((double)a, &sd, &cd);
      s = (T)sd;
      c = (T)cd;
    }
    if (!inverse) {
      c1 = (T(1) - c) / a2;
      c2 = (T(1) - s / a) / a2;
    } else {
      c1 = T(-0.5);
      c2 = T(1) / a2 - (T(1) + c) / (T(2) * a * s);
    }
  }
  // S = [th]x, S^2 = th th^T - |th|^2 I
  T S[9] = {T(0), -th[2], th[1], th[2], T(0), -th[0], -th[1], th[0], T(0)};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      M[3 * i + j] = (i == j ? T(1) : T(0)) + c1 * S[3 * i + j] + c2 * (th[i] * th[j] - (i == j ? a2 : T(0)));
}

template <typename T>
XK_D void mm3(const T* A, const T* B, T* C) {  // C = A B
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}
template <typename T>
XK_D void mtm3(const T* A, const T* B, T* C) {  // C = A^T B
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[3 * i + j] = A[i] * B[j] + A[3 + i] * B[3 + j] + A[6 + i] * B[6 + j];
}

// Local Timoshenko stiffness coefficients of one element (_beam_cr.py:911-998).
template <typename T>
struct KeCoef {
  T ea, gj, k3y, k2y, k1ay, k1by, k3z, k2z, k1az, k1bz;
};

template <typename T>
XK_D KeCoef<T> ke_coef(const xk_section& s, T L0) {
  T L = L0;
  T iL = T(1) / L;
  T E = (T)s.E, G = (T)s.G, A = (T)s.A, Iy = (T)s.Iy, Iz = (T)s.Iz, J = (T)s.J;
  T phy = T(12) * E * Iy / ((T)s.kappa_y * G * A * L * L);
  T phz = T(12) * E * Iz / ((T)s.kappa_z * G * A * L * L);
  if (s.scf > 0.0) {
    T sc = (T)s.scf;
    phy = phy / (T(1) + sc * L * L * A / (T(12) * Iy));
    phz = phz / (T(1) + sc * L * L * A / (T(12) * Iz));
  }
  KeCoef<T> k;
  k.ea = E * A * iL;
  k.gj = G * J * iL;
  T dy = T(1) / (T(1) + phy), dz = T(1) / (T(1) + phz);
  T eiy = E * Iy * iL, eiz = E * Iz * iL;
  k.k3y = T(12) * eiy * iL * iL * dy;
  k.k2y = T(6) * eiy * iL * dy;
  k.k1ay = (T(4) + phy) * eiy * dy;
  k.k1by = (T(2) - phy) * eiy * dy;
  k.k3z = T(12) * eiz * iL * iL * dz;
  k.k2z = T(6) * eiz * iL * dz;
  k.k1az = (T(4) + phz) * eiz * dz;
  k.k1bz = (T(2) - phz) * eiz * dz;
  return k;
}

// Entry (i, j) of the local stiffness; zeros fold away after unrolling.
template <typename T>
XK_D T kev(const KeCoef<T>& k, int i, int j) {
  switch (i) {
    case 0: return j == 0 ? k.ea : (j == 6 ? -k.ea : T(0));
    case 6: return j == 0 ? -k.ea : (j == 6 ? k.ea : T(0));
    case 3: return j == 3 ? k.gj : (j == 9 ? -k.gj : T(0));
    case 9: return j == 3 ? -k.gj : (j == 9 ? k.gj : T(0));
    case 1: return j == 1 ? k.k3z : j == 5 ? k.k2z : j == 7 ? -k.k3z : j == 11 ? k.k2z : T(0);
    case 5: return j == 1 ? k.k2z : j == 5 ? k.k1az : j == 7 ? -k.k2z : j == 11 ? k.k1bz : T(0);
    case 7: return j == 1 ? -k.k3z : j == 5 ? -k.k2z : j == 7 ? k.k3z : j == 11 ? -k.k2z : T(0);
    case 11: return j == 1 ? k.k2z : j == 5 ? k.k1bz : j == 7 ? -k.k2z : j == 11 ? k.k1az : T(0);
    case 2: return j == 2 ? k.k3y : j == 4 ? -k.k2y : j == 8 ? -k.k3y : j == 10 ? -k.k2y : T(0);
    case 4: return j == 2 ? -k.k2y : j == 4 ? k.k1ay : j == 8 ? k.k2y : j == 10 ? k.k1by : T(0);
    case 8: return j == 2 ? -k.k3y : j == 4 ? k.k2y : j == 8 ? k.k3y : j == 10 ? k.k2y : T(0);
    case 10: return j == 2 ? -k.k2y : j == 4 ? k.k1by : j == 8 ? k.k2y : j == 10 ? k.k1ay : T(0);
  }
  return T(0);
}

__global__ void k_beam_reference(xk_mesh m, double vx, double vy, double vz, int has_vref,
                                 double* __restrict__ ref) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.n_elems) return;
  const long long ne = m.n_elems;
  int a = m.conn[2 * e], b = m.conn[2 * e + 1];
  double d[3];
  for (int i = 0; i < 3; ++i) d[i] = m.X[3 * b + i] - m.X[3 * a + i];
  double L = sqrt(xdot_seq(d, d));
  double ex[3] = {d[0] / L, d[1] / L, d[2] / L};
  double vr[3] = {vx, vy, vz};
  if (!has_vref) {
    double a0 = fabs(ex[0]), a1 = fabs(ex[1]), a2 = fabs(ex[2]);
    vr[0] = vr[1] = vr[2] = 0.0;
    vr[(a0 <= a1 && a0 <= a2) ? 0 : (a1 <= a2 ? 1 : 2)] = 1.0;
  }
  double ez[3], ey[3];
  cross3(ex, vr, ez);
  double nz = sqrt(xdot_seq(ez, ez));
  if (nz < 1e-10) nz = 1e-10;
  for (int i = 0; i < 3; ++i) ez[i] /= nz;
  cross3(ez, ex, ey);
  ref[0 * ne + e] = L;
  for (int i = 0; i < 3; ++i) {
    ref[(1 + i) * ne + e] = ex[i];
    ref[(4 + i) * ne + e] = ey[i];
    ref[(7 + i) * ne + e] = ez[i];
  }
}

// Local forces, global element force and the symmetrised analytic tangent
// (_beam_assembly.py:265-323) from the corotated frame R_cr, the deformed axis
// ex, 1/L, the local rotations t1, t2, the nodal rotation vectors tha, thb and
// the axial stretch dax, written into f_int rows and the four 6x6 blocks.
template <typename T>
XK_D void beam_tail(const KeCoef<T>& kc, const T* Rcr, const T* ex, T iL, const T* t1, const T* t2, const T* tha,
                    const T* thb, T dax, int a, int b, int e, uint8_t fl, const int32_t* __restrict__ blk,
                    double* __restrict__ f_int, T* __restrict__ Kv) {
  T fcr[12];
  fcr[0] = -kc.ea * dax;
  fcr[1] = kc.k2z * (t1[2] + t2[2]);
  fcr[2] = -kc.k2y * (t1[1] + t2[1]);
  fcr[3] = kc.gj * (t1[0] - t2[0]);
  fcr[4] = kc.k1ay * t1[1] + kc.k1by * t2[1];
  fcr[5] = kc.k1az * t1[2] + kc.k1bz * t2[2];
  fcr[6] = kc.ea * dax;
  fcr[7] = -fcr[1];
  fcr[8] = -fcr[2];
  fcr[9] = -fcr[3];
  fcr[10] = kc.k1by * t1[1] + kc.k1ay * t2[1];
  fcr[11] = kc.k1bz * t1[2] + kc.k1az * t2[2];
  if (f_int) {
#pragma unroll
    for (int blkI = 0; blkI < 4; ++blkI) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        double v = (double)(Rcr[i] * fcr[3 * blkI] + Rcr[3 + i] * fcr[3 * blkI + 1] + Rcr[6 + i] * fcr[3 * blkI + 2]);
        long long dof = (blkI < 2 ? 6LL * a : 6LL * b) + 3 * (blkI & 1) + i;
        bool fw = (blkI < 2) ? (fl & 1) : (fl & 8);
        if (fw) f_int[dof] = v; else f_int[dof] += v;
      }
    }
  }
  if (!Kv) return;
  // ------------------------------------------------ tangent
  T Sx[9] = {T(0), -ex[2], ex[1], ex[2], T(0), -ex[0], -ex[1], ex[0], T(0)};
  T dpsi[9];
  mm3(Rcr, Sx, dpsi);
#pragma unroll
  for (int i = 0; i < 9; ++i) dpsi[i] *= iL;
  T P1[9], Q1[9], P2[9], Q2[9];
  {
    T Ti[9], Ts[9], tmp[9];
    tangent_ops<T>(t1, true, Ti);
    mm3(Ti, dpsi, P1);
    tangent_ops<T>(tha, false, Ts);
    mm3(Ti, Rcr, tmp);
    mm3(tmp, Ts, Q1);
    tangent_ops<T>(t2, true, Ti);
    mm3(Ti, dpsi, P2);
    tangent_ops<T>(thb, false, Ts);
    mm3(Ti, Rcr, tmp);
    mm3(tmp, Ts, Q2);
  }
  // unsymmetrised block rows I: [G_I, H_I, -G_I, J_I]
  T Gm[4][9], Hm[4][9], Jm[4][9];
#pragma unroll
  for (int I = 0; I < 4; ++I) {
    T A[9], Hl[9], Jl[9];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const int row = 3 * I + r;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        T acc = -kev(kc, row, 6) * ex[c];
        T h = T(0), jj = T(0);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          acc += kev(kc, row, 3 + q) * P1[3 * q + c] + kev(kc, row, 9 + q) * P2[3 * q + c];
          h += kev(kc, row, 3 + q) * Q1[3 * q + c];
          jj += kev(kc, row, 9 + q) * Q2[3 * q + c];
        }
        A[3 * r + c] = acc;
        Hl[3 * r + c] = h;
        Jl[3 * r + c] = jj;
      }
    }
    // + [f_I]x dpsi
    const T f0 = fcr[3 * I], f1 = fcr[3 * I + 1], f2 = fcr[3 * I + 2];
    T Sf[9] = {T(0), -f2, f1, f2, T(0), -f0, -f1, f0, T(0)};
    T SfD[9];
    mm3(Sf, dpsi, SfD);
#pragma unroll
    for (int i = 0; i < 9; ++i) A[i] += SfD[i];
    mtm3(Rcr, A, Gm[I]);
    mtm3(Rcr, Hl, Hm[I]);
    mtm3(Rcr, Jl, Jm[I]);
  }
  // symmetrise and write the stored 6x6 node blocks (the off-diagonal block below the diagonal,
  // id -1, is the transpose of the stored one)
#pragma unroll
  for (int nb = 0; nb < 4; ++nb) {  // 0 aa, 1 ab, 2 ba, 3 bb
    const int I0 = (nb >> 1) * 2, J0 = (nb & 1) * 2;
    const int bi = blk[4LL * e + nb];
    if (bi < 0) continue;
    T* dst = Kv + 36LL * bi;
    const bool fw = (fl >> nb) & 1;
#pragma unroll
    for (int ii = 0; ii < 2; ++ii)
#pragma unroll
      for (int jj = 0; jj < 2; ++jj) {
        const int I = I0 + ii, J = J0 + jj;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            T xij = (J == 0) ? Gm[I][3 * r + c] : (J == 1) ? Hm[I][3 * r + c] : (J == 2) ? -Gm[I][3 * r + c] : Jm[I][3 * r + c];
            T xji = (I == 0) ? Gm[J][3 * c + r] : (I == 1) ? Hm[J][3 * c + r] : (I == 2) ? -Gm[J][3 * c + r] : Jm[J][3 * c + r];
            T v = T(0.5) * (xij + xji);
            const int idx = (3 * ii + r) * 6 + 3 * jj + c;
            if (fw) dst[idx] = v; else dst[idx] += v;
          }
      }
  }
}


template <int P>
__global__ void __launch_bounds__(BEAM_T) k_beam(xk_mesh m, xk_section sec, const double* __restrict__ ref,
                                                 const int32_t* __restrict__ order, int k0, int k1,
                                                 const int32_t* __restrict__ blk, const uint8_t* __restrict__ first,
                                                 const double* __restrict__ u, double* __restrict__ f_int,
                                                 typename Prec<P>::T* __restrict__ Kv) {
  typedef typename Prec<P>::T T;
  int k = k0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= k1) return;
  const int e = order[k];
  const long long ne = m.n_elems;
  const int a = m.conn[2 * e], b = m.conn[2 * e + 1];
  // ------------------------------------------------ double: frame and strain
  const double L0 = ref[e];
  double R0[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) R0[i] = ref[(1 + i) * ne + e];
  double ua[6], ub[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) { ua[i] = u[6LL * a + i]; ub[i] = u[6LL * b + i]; }
  double dxd[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) dxd[i] = (m.X[3LL * b + i] + ub[i]) - (m.X[3LL * a + i] + ua[i]);
  const double Ld = sqrt(dot3(dxd, dxd));
  const double iLd = 1.0 / Ld;
  double exd[3] = {dxd[0] * iLd, dxd[1] * iLd, dxd[2] * iLd};
  double qr[4];
  quat_between(R0, exd, qr);  // R0 row 0 is e_x of the reference frame
  double qrc[4] = {qr[0], -qr[1], -qr[2], -qr[3]};
  double th1[3], th2[3];
  {
    double qn[4], qx[4], tx[3];
    quat_of_rotvec(ua + 3, qn);
    qmul(qrc, qn, qx);
    rotvec_of_quat(qx, tx);
#pragma unroll
    for (int i = 0; i < 3; ++i) th1[i] = R0[3 * i] * tx[0] + R0[3 * i + 1] * tx[1] + R0[3 * i + 2] * tx[2];
    quat_of_rotvec(ub + 3, qn);
    qmul(qrc, qn, qx);
    rotvec_of_quat(qx, tx);
#pragma unroll
    for (int i = 0; i < 3; ++i) th2[i] = R0[3 * i] * tx[0] + R0[3 * i + 1] * tx[1] + R0[3 * i + 2] * tx[2];
  }
  const T dax = (T)(Ld - L0);
  T Rrod[9], Rcr[9], R0t[9];
  rotmat_of_quat<T>(qr, Rrod);
#pragma unroll
  for (int i = 0; i < 9; ++i) R0t[i] = (T)R0[i];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      Rcr[3 * i + j] = R0t[3 * i] * Rrod[3 * j] + R0t[3 * i + 1] * Rrod[3 * j + 1] + R0t[3 * i + 2] * Rrod[3 * j + 2];
  const T t1[3] = {(T)th1[0], (T)th1[1], (T)th1[2]};
  const T t2[3] = {(T)th2[0], (T)th2[1], (T)th2[2]};
  const T ex[3] = {(T)exd[0], (T)exd[1], (T)exd[2]};
  const T tha[3] = {(T)ua[3], (T)ua[4], (T)ua[5]};
  const T thb[3] = {(T)ub[3], (T)ub[4], (T)ub[5]};
  beam_tail<T>(ke_coef<T>(sec, (T)L0), Rcr, ex, (T)iLd, t1, t2, tha, thb, dax, a, b, e, first[e], blk, f_int, Kv);
}

// Mixed path: every operation in float.  With Delta u = u_b - u_a and the
// reference chord dx0 (e0 = dx0 / L0):
//   L - L0        = Delta u . (2 dx0 + Delta u) / (L + L0)
//   e0 x e        = e0 x Delta u / L          (e0 x dx0 = 0)
//   1 + e0 . e    = (L + L0 + e0 . Delta u) / L
// none of which cancels, so the corotated frame keeps float accuracy relative
// to the (small) deformation instead of to the coordinates.
struct Frame32 {
  float Rcr[9], exd[3], iLd, th1[3], th2[3], tha[3], thb[3], dax, L0;
};

// The local rotations th1 (node a) and th2 (node b) each take a quaternion log map: a lane of a
// quad computes the one of its node (lanes 0, 1: a; lanes 2, 3: b) and takes the other from the
// lane two places away, so every lane ends with both.
XK_D void frame32(const float* __restrict__ E, const float* __restrict__ NA, const float* __restrict__ NB, Frame32& F,
                  int lane_in_quad) {
  const float dx0[3] = {E[0], E[1], E[2]};
  F.L0 = E[3];
  float R0[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) R0[i] = E[4 + i];
  float ua[6], ub[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) { ua[i] = NA[i]; ub[i] = NB[i]; }
  const float du[3] = {ub[0] - ua[0], ub[1] - ua[1], ub[2] - ua[2]};
  const float dxd[3] = {dx0[0] + du[0], dx0[1] + du[1], dx0[2] + du[2]};
  const float Ld = sqrtf(dot3(dxd, dxd));
  const float iLd = 1.0f / Ld;
  F.iLd = iLd;
  const float two_dx_du[3] = {2.0f * dx0[0] + du[0], 2.0f * dx0[1] + du[1], 2.0f * dx0[2] + du[2]};
  F.dax = dot3(du, two_dx_du) / (Ld + F.L0);
  for (int i = 0; i < 3; ++i) F.exd[i] = dxd[i] * iLd;
  float qr[4];
  {
    float v[3];
    cross3(R0, du, v);
    const float opc = fmaxf((Ld + F.L0 + dot3(R0, du)) * iLd, 1e-12f);
    const float w = sqrtf(0.5f * opc);
    const float kk = 0.5f * iLd / w;
    qr[0] = w; qr[1] = kk * v[0]; qr[2] = kk * v[1]; qr[3] = kk * v[2];
  }
  const float qrc[4] = {qr[0], -qr[1], -qr[2], -qr[3]};
  {
    const bool node_b = lane_in_quad >= 2;
    float th[3], qn[4], qx[4], tx[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) th[i] = node_b ? ub[3 + i] : ua[3 + i];
    quat_of_rotvecf(th, qn);
    qmulf(qrc, qn, qx);
    rotvec_of_quatf(qx, tx);
    float mine[3], other[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      mine[i] = R0[3 * i] * tx[0] + R0[3 * i + 1] * tx[1] + R0[3 * i + 2] * tx[2];
      other[i] = __shfl_xor_sync(0xffffffffu, mine[i], 2);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      F.th1[i] = node_b ? other[i] : mine[i];
      F.th2[i] = node_b ? mine[i] : other[i];
    }
  }
  for (int i = 0; i < 3; ++i) { F.tha[i] = ua[3 + i]; F.thb[i] = ub[3 + i]; }
  float Rrod[9];
  {
    const float w = qr[0], x = qr[1], y = qr[2], z = qr[3];
    Rrod[0] = 1.f - 2.f * (y * y + z * z); Rrod[1] = 2.f * (x * y - w * z); Rrod[2] = 2.f * (x * z + w * y);
    Rrod[3] = 2.f * (x * y + w * z); Rrod[4] = 1.f - 2.f * (x * x + z * z); Rrod[5] = 2.f * (y * z - w * x);
    Rrod[6] = 2.f * (x * z - w * y); Rrod[7] = 2.f * (y * z + w * x); Rrod[8] = 1.f - 2.f * (x * x + y * y);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      F.Rcr[3 * i + j] = R0[3 * i] * Rrod[3 * j] + R0[3 * i + 1] * Rrod[3 * j + 1] + R0[3 * i + 2] * Rrod[3 * j + 2];
}

// Mixed path, four lanes per element: lane I of a quad computes block row I of
// the unsymmetrised tangent ([G_I, H_I, -G_I, J_I], see beam_tail) and the f
// rows of DOF group I; the quad exchanges the rows through shared memory to
// symmetrise, and lane I stores rows 3I..3I+2 of the 12x12 element tangent.
//
// CHAIN: all elements in one launch (order == NULL: element k is element k),
// for meshes in which every node has at most two elements and no two
// elements share both nodes (wires).  The node rows of f_int and the diagonal
// blocks, which two elements share, are zeroed first (k_beam_zero32) and
// receive their two contributions by atomic adds; 0 + a + b = 0 + b + a, so
// the result does not depend on their order.  The off-diagonal blocks have one
// writer each.  Otherwise the launch covers one colour of the plan.
constexpr int BEAMQ_T = 128;

template <bool CHAIN>
__global__ void __launch_bounds__(BEAMQ_T, 7) k_beam32q(xk_mesh m, xk_section sec, const float* __restrict__ e32,
                                                     const int32_t* __restrict__ order, int k0, int k1,
                                                     const int32_t* __restrict__ blk,
                                                     const uint8_t* __restrict__ first, const float* __restrict__ n32,
                                                     double* __restrict__ f_int, float* __restrict__ Kv) {
  __shared__ float sx[BEAMQ_T / 4][4][27];
  // the element's three stored 6x6 blocks, staged: aa, the off-diagonal one above the diagonal, bb
  __shared__ __align__(16) float kst[BEAMQ_T / 4][3][36];
  __shared__ int s_e[BEAMQ_T / 4];
  const int q = threadIdx.x >> 2, I = threadIdx.x & 3;
  const int k = k0 + blockIdx.x * (BEAMQ_T / 4) + q;
  const bool live = k < k1;
  const int e = CHAIN ? (live ? k : k0) : (live ? order[k] : order[k0]);
  if (I == 0) s_e[q] = live ? e : -1;
  const int a = m.conn[2 * e], b = m.conn[2 * e + 1];
  Frame32 F;
  frame32(e32 + (long long)e * XK_ELEM32_STRIDE, n32 + (long long)a * XK_NODE32_STRIDE + 6,
          n32 + (long long)b * XK_NODE32_STRIDE + 6, F, I);
  const KeCoef<float> kc = ke_coef<float>(sec, F.L0);
  const float* t1 = F.th1;
  const float* t2 = F.th2;
  float fcr[12];
  fcr[0] = -kc.ea * F.dax;
  fcr[1] = kc.k2z * (t1[2] + t2[2]);
  fcr[2] = -kc.k2y * (t1[1] + t2[1]);
  fcr[3] = kc.gj * (t1[0] - t2[0]);
  fcr[4] = kc.k1ay * t1[1] + kc.k1by * t2[1];
  fcr[5] = kc.k1az * t1[2] + kc.k1bz * t2[2];
  fcr[6] = kc.ea * F.dax;
  fcr[7] = -fcr[1];
  fcr[8] = -fcr[2];
  fcr[9] = -fcr[3];
  fcr[10] = kc.k1by * t1[1] + kc.k1ay * t2[1];
  fcr[11] = kc.k1bz * t1[2] + kc.k1az * t2[2];
  const float* Rcr = F.Rcr;
  const uint8_t fl = first[e];
  if (live && f_int) {
    const float g0 = I == 0 ? fcr[0] : I == 1 ? fcr[3] : I == 2 ? fcr[6] : fcr[9];
    const float g1 = I == 0 ? fcr[1] : I == 1 ? fcr[4] : I == 2 ? fcr[7] : fcr[10];
    const float g2 = I == 0 ? fcr[2] : I == 1 ? fcr[5] : I == 2 ? fcr[8] : fcr[11];
    for (int i = 0; i < 3; ++i) {
      const double v = (double)(Rcr[i] * g0 + Rcr[3 + i] * g1 + Rcr[6 + i] * g2);
      const long long dof = (I < 2 ? 6LL * a : 6LL * b) + 3 * (I & 1) + i;
      const bool fw = (I < 2) ? (fl & 1) : (fl & 8);
      if (CHAIN) atomicAdd(f_int + dof, v);
      else if (fw) f_int[dof] = v;
      else f_int[dof] += v;
    }
  }
  if (!Kv) return;  // uniform over the launch
  const float* ex = F.exd;
  float dpsi[9];
  {
    const float Sx[9] = {0.f, -ex[2], ex[1], ex[2], 0.f, -ex[0], -ex[1], ex[0], 0.f};
    mm3(Rcr, Sx, dpsi);
#pragma unroll
    for (int i = 0; i < 9; ++i) dpsi[i] *= F.iLd;
  }
  // P1 = T^-1(t1) dpsi, Q1 = T^-1(t1) Rcr T(tha), P2, Q2 likewise at node b are needed by all
  // rows (Ke_{I1} and Ke_{I3}); lane I computes the I-th of (P1, Q1, P2, Q2) and the quad shares
  // them through shared memory
  {
    float thi[3], Ti[9], X[9];
#pragma unroll
    for (int c = 0; c < 3; ++c) thi[c] = I < 2 ? t1[c] : t2[c];
    tangent_ops<float>(thi, true, Ti);
    if (I & 1) {
      float thn[3], Ts[9], tmp[9];
#pragma unroll
      for (int c = 0; c < 3; ++c) thn[c] = I < 2 ? F.tha[c] : F.thb[c];
      tangent_ops<float>(thn, false, Ts);
      mm3(Ti, Rcr, tmp);
      mm3(tmp, Ts, X);
    } else {
      mm3(Ti, dpsi, X);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) sx[q][I][i] = X[i];
  }
  __syncwarp();
  const float* P1 = sx[q][0];
  const float* Q1 = sx[q][1];
  const float* P2 = sx[q][2];
  const float* Q2 = sx[q][3];
  // block row I of the local stiffness against the theta1 (K1), theta2 (K3) and
  // axial (k6) columns, built with selects so that the quad does not diverge
  const bool i0 = I == 0, i1 = I == 1, i2 = I == 2;
  float K1[9], K3[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) { K1[i] = 0.f; K3[i] = 0.f; }
  const float tz = i0 ? kc.k2z : -kc.k2z, ty = i0 ? -kc.k2y : kc.k2y;  // rows of I = 0 / 2
  const bool trans = i0 || i2;
  K1[5] = trans ? tz : 0.f;
  K3[5] = K1[5];
  K1[7] = trans ? ty : 0.f;
  K3[7] = K1[7];
  K1[0] = trans ? 0.f : (i1 ? kc.gj : -kc.gj);
  K3[0] = -K1[0];
  K1[4] = trans ? 0.f : (i1 ? kc.k1ay : kc.k1by);
  K3[4] = trans ? 0.f : (i1 ? kc.k1by : kc.k1ay);
  K1[8] = trans ? 0.f : (i1 ? kc.k1az : kc.k1bz);
  K3[8] = trans ? 0.f : (i1 ? kc.k1bz : kc.k1az);
  const float k6 = i0 ? -kc.ea : (i2 ? kc.ea : 0.f);  // only row 3I of the block
  const float fI0 = i0 ? fcr[0] : i1 ? fcr[3] : i2 ? fcr[6] : fcr[9];
  const float fI1 = i0 ? fcr[1] : i1 ? fcr[4] : i2 ? fcr[7] : fcr[10];
  const float fI2 = i0 ? fcr[2] : i1 ? fcr[5] : i2 ? fcr[8] : fcr[11];
  float G[9], H[9], J[9];
  {
    float A[9], Hl[9], Jl[9];
    mm3(K1, P1, A);
    float tmp[9];
    mm3(K3, P2, tmp);
#pragma unroll
    for (int i = 0; i < 9; ++i) A[i] += tmp[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) A[c] -= k6 * ex[c];
    mm3(K1, Q1, Hl);
    mm3(K3, Q2, Jl);
    const float Sf[9] = {0.f, -fI2, fI1, fI2, 0.f, -fI0, -fI1, fI0, 0.f};
    float SfD[9];
    mm3(Sf, dpsi, SfD);
#pragma unroll
    for (int i = 0; i < 9; ++i) A[i] += SfD[i];
    mtm3(Rcr, A, G);
    mtm3(Rcr, Hl, H);
    mtm3(Rcr, Jl, J);
  }
  __syncwarp();  // every lane has read P1..Q2 before sx is overwritten
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    sx[q][I][i] = G[i];
    sx[q][I][9 + i] = H[i];
    sx[q][I][18 + i] = J[i];
  }
  __syncwarp();
  // row I of the symmetrised tangent: Ks[I][Jb] = (X_IJb + X_JbI^T) / 2 with
  // X_I0 = G_I, X_I1 = H_I, X_I2 = -G_I, X_I3 = J_I, staged per stored block (the off-diagonal
  // block below the diagonal, ba for a < b and ab for a > b, is the transpose of the other)
  const int nb_lower = a < b ? 2 : 1;
#pragma unroll
  for (int Jb = 0; Jb < 4; ++Jb) {
    const int nb = (I >> 1) * 2 + (Jb >> 1);  // 0 aa, 1 ab, 2 ba, 3 bb
    if (nb == nb_lower) continue;
    const int slot = nb == 0 ? 0 : (nb == 3 ? 2 : 1);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float xij = (Jb == 0) ? G[3 * r + c] : (Jb == 1) ? H[3 * r + c] : (Jb == 2) ? -G[3 * r + c] : J[3 * r + c];
        const float* o = sx[q][Jb];
        const int off = i1 ? 9 : ((I == 3) ? 18 : 0);
        const float xji = (i2 ? -1.f : 1.f) * o[off + 3 * c + r];
        kst[q][slot][(3 * (I & 1) + r) * 6 + 3 * (Jb & 1) + c] = 0.5f * (xij + xji);
      }
  }
  __syncwarp();
  // the warp's 8 elements x 3 stored blocks as 9 float4 per block (a block starts at 144 B * index),
  // first writer of a block stores, later colours add
  const int lane = threadIdx.x & 31, q0 = (threadIdx.x >> 5) * 8;
  for (int t = lane; t < 8 * 3 * 9; t += 32) {
    const int qq = q0 + t / 27, slot = (t % 27) / 9, ch = t % 9;
    const int ee = s_e[qq];
    if (ee < 0) continue;
    const int nb = slot == 0 ? 0 : (slot == 2 ? 3 : (blk[4LL * ee + 1] >= 0 ? 1 : 2));
    const int bi = blk[4LL * ee + nb];
    const float4 v = reinterpret_cast<const float4*>(kst[qq][slot])[ch];
    float4* dst = reinterpret_cast<float4*>(Kv + 36LL * bi) + ch;
    if (CHAIN) {
      if (nb == 0 || nb == 3) atomicAdd(dst, v);  // diagonal block, shared with the neighbour element
      else *dst = v;
    } else if ((first[ee] >> nb) & 1) {
      *dst = v;
    } else {
      float4 o = *dst;
      o.x += v.x; o.y += v.y; o.z += v.z; o.w += v.w;
      *dst = o;
    }
  }
}

// Chain launches: zero the node rows of f_int and the diagonal blocks that the elements add into,
// one thread per 16 bytes (nine per 6x6 float block, three per node row of f_int), so that
// neighbouring threads write neighbouring bytes.
__global__ void k_beam_zero32(int n_nodes, const int32_t* __restrict__ node_diag, double* __restrict__ f_int,
                              float* __restrict__ Kv) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  if (Kv && t < 9LL * n_nodes) {
    const int d = node_diag[t / 9];
    if (d >= 0) reinterpret_cast<float4*>(Kv + 36LL * d)[t % 9] = z;  // no element at the node: not written
  }
  if (f_int && t < 3LL * n_nodes && node_diag[t / 3] >= 0) {
    if (((uintptr_t)f_int & 15) == 0) {
      reinterpret_cast<float4*>(f_int)[t] = z;
    } else {
      f_int[2 * t] = 0.0;
      f_int[2 * t + 1] = 0.0;
    }
  }
}

__global__ void k_beam_prepare32(xk_mesh m, const double* __restrict__ ref, float* __restrict__ e32) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.n_elems) return;
  const long long ne = m.n_elems;
  const int a = m.conn[2 * e], b = m.conn[2 * e + 1];
  float* E = e32 + (long long)e * XK_ELEM32_STRIDE;
  for (int i = 0; i < 3; ++i) E[i] = (float)(m.X[3LL * b + i] - m.X[3LL * a + i]);
  E[3] = (float)ref[e];
  for (int i = 0; i < 9; ++i) E[4 + i] = (float)ref[(1 + i) * ne + e];
  const double r = m.radii[e];
  const float rh = (float)r;
  E[13] = rh;
  E[14] = (float)(r - (double)rh);
  E[15] = 0.0f;
}

__global__ void k_lumped_mass(xk_mesh m, xk_section sec, double rho, const int32_t* __restrict__ order, int k0,
                              int k1, const uint8_t* __restrict__ first, double* __restrict__ out) {
  int k = k0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= k1) return;
  int e = order[k];
  int a = m.conn[2 * e], b = m.conn[2 * e + 1];
  double d[3];
  for (int i = 0; i < 3; ++i) d[i] = m.X[3 * b + i] - m.X[3 * a + i];
  double L = sqrt(xdot_seq(d, d));
  double mm = rho * sec.A * L;
  double mt = rho * (sec.Iy + sec.Iz) * L;
  double ri = mm * L * L / 78.0;
  double v[6] = {mm / 2.0, mm / 2.0, mm / 2.0, mt / 2.0, ri, ri};
  uint8_t fl = first[e];
  for (int i = 0; i < 6; ++i) {
    if (fl & 1) out[6LL * a + i] = v[i]; else out[6LL * a + i] += v[i];
    if (fl & 8) out[6LL * b + i] = v[i]; else out[6LL * b + i] += v[i];
  }
}

}  // namespace

extern "C" xk_status xk_beam_reference(const xk_mesh* m, const double* v_ref, double* elem_ref, xk_stream s) {
  if (!m || !elem_ref) return xk_set_error(XK_ERR_ARG, "xk_beam_reference: null argument");
  if (m->n_elems == 0) return XK_OK;
  double vr[3] = {0.0, 0.0, 0.0};
  if (v_ref) { vr[0] = v_ref[0]; vr[1] = v_ref[1]; vr[2] = v_ref[2]; }
  k_beam_reference<<<xk_blocks(m->n_elems, 256), 256, 0, (cudaStream_t)s>>>(*m, vr[0], vr[1], vr[2], v_ref != nullptr,
                                                                            elem_ref);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_beam_assemble(const xk_mesh* m, const xk_section* sec, const double* elem_ref,
                                      const xk_beam_plan* plan, const double* u, int precision, double* f_int,
                                      void* K_vals, xk_stream s) {
  if (!m || !sec || !elem_ref || !plan || !u) return xk_set_error(XK_ERR_ARG, "xk_beam_assemble: null argument");
  if (precision != XK_FP64 && precision != XK_MIXED) return xk_set_error(XK_ERR_ARG, "xk_beam_assemble: precision");
  if (!f_int && !K_vals) return XK_OK;
  cudaStream_t st = (cudaStream_t)s;
  for (int c = 0; c < plan->n_colors; ++c) {
    int k0 = plan->color_ptr_host[c], k1 = plan->color_ptr_host[c + 1];
    if (k1 <= k0) continue;
    int nb = xk_blocks(k1 - k0, BEAM_T);
    if (precision == XK_FP64)
      k_beam<XK_FP64><<<nb, BEAM_T, 0, st>>>(*m, *sec, elem_ref, plan->elem_order, k0, k1, plan->blk, plan->first, u,
                                              f_int, (double*)K_vals);
    else
      k_beam<XK_MIXED><<<nb, BEAM_T, 0, st>>>(*m, *sec, elem_ref, plan->elem_order, k0, k1, plan->blk, plan->first, u,
                                               f_int, (float*)K_vals);
    XK_CHECK_LAUNCH();
  }
  return XK_OK;
}

extern "C" xk_status xk_beam_lumped_mass(const xk_mesh* m, const xk_section* sec, const xk_beam_plan* plan,
                                         double rho, double* out, xk_stream s) {
  if (!m || !sec || !plan || !out) return xk_set_error(XK_ERR_ARG, "xk_beam_lumped_mass: null argument");
  for (int c = 0; c < plan->n_colors; ++c) {
    int k0 = plan->color_ptr_host[c], k1 = plan->color_ptr_host[c + 1];
    if (k1 <= k0) continue;
    k_lumped_mass<<<xk_blocks(k1 - k0, 256), 256, 0, (cudaStream_t)s>>>(*m, *sec, rho, plan->elem_order, k0, k1,
                                                                         plan->first, out);
    XK_CHECK_LAUNCH();
  }
  return XK_OK;
}

extern "C" xk_status xk_beam_prepare32(const xk_mesh* m, const double* elem_ref, float* elem32, xk_stream s) {
  if (!m || !elem_ref || !elem32) return xk_set_error(XK_ERR_ARG, "xk_beam_prepare32: null argument");
  if (m->n_elems == 0) return XK_OK;
  k_beam_prepare32<<<xk_blocks(m->n_elems, 256), 256, 0, (cudaStream_t)s>>>(*m, elem_ref, elem32);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_beam_assemble32(const xk_mesh* m, const xk_section* sec, const float* elem32,
                                        const xk_beam_plan* plan, const float* node32, double* f_int, float* K_vals,
                                        xk_stream s) {
  if (!m || !sec || !elem32 || !plan || !node32) return xk_set_error(XK_ERR_ARG, "xk_beam_assemble32: null argument");
  if (!f_int && !K_vals) return XK_OK;
  cudaStream_t st = (cudaStream_t)s;
  if (plan->node_diag) {  // chain mesh: one launch over all elements
    if (m->n_elems == 0) return XK_OK;
    k_beam_zero32<<<xk_blocks(9LL * m->n_nodes, 256), 256, 0, st>>>(m->n_nodes, plan->node_diag, f_int, K_vals);
    k_beam32q<true><<<xk_blocks(4LL * m->n_elems, BEAMQ_T), BEAMQ_T, 0, st>>>(
        *m, *sec, elem32, nullptr, 0, m->n_elems, plan->blk, plan->first, node32, f_int, K_vals);
    XK_CHECK_LAUNCH();
    return XK_OK;
  }
  for (int c = 0; c < plan->n_colors; ++c) {
    const int k0 = plan->color_ptr_host[c], k1 = plan->color_ptr_host[c + 1];
    if (k1 <= k0) continue;
    k_beam32q<false><<<xk_blocks(4LL * (k1 - k0), BEAMQ_T), BEAMQ_T, 0, st>>>(
        *m, *sec, elem32, plan->elem_order, k0, k1, plan->blk, plan->first, node32, f_int, K_vals);
    XK_CHECK_LAUNCH();
  }
  return XK_OK;
}
