// Corotational Timoshenko beam: internal force and analytic tangent per element.
//
// Mirrors _assemble_cr_beam3d_batch_impl (xkep_cae/elements/_beam_assembly.py:211-325)
// one element per thread, with the corotated frame in quaternion form:
//   R_cr = R0 R_rod^T,  theta_def = log(R_cr R_node R0^T) = R0 log(q_rod^* (x) q_node)
// which equals the reference's matrix Shepperd route for rotations below pi.
// k_beam<P> (xk_beam_assemble) takes the frame in double in both precision modes
// and runs everything downstream of it (local stiffness, f_cr, B, K_mat, K_geo)
// in Prec<P>::T; k_beam32e (xk_beam_assemble32, the mixed engine) runs all of it
// in float from the prepared element and node records.
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

// A section value in the element's precision; to float in integer arithmetic (the conversion instruction
// issues at the FP64 rate), the same bits as the cast.
template <typename T>
XK_D T sec_val(double x);
template <>
XK_D double sec_val<double>(double x) { return x; }
template <>
XK_D float sec_val<float>(double x) { return xk_d2f(x); }

template <typename T>
XK_D KeCoef<T> ke_coef(const xk_section& s, T L0) {
  T L = L0;
  T iL = T(1) / L;
  T E = sec_val<T>(s.E), G = sec_val<T>(s.G), A = sec_val<T>(s.A), Iy = sec_val<T>(s.Iy), Iz = sec_val<T>(s.Iz),
    J = sec_val<T>(s.J);
  T phy = T(12) * E * Iy / (sec_val<T>(s.kappa_y) * G * A * L * L);
  T phz = T(12) * E * Iz / (sec_val<T>(s.kappa_z) * G * A * L * L);
  if (__double_as_longlong(s.scf) > 0 && __double_as_longlong(s.scf) <= 0x7ff0000000000000LL) {  // scf > 0
    T sc = sec_val<T>(s.scf);
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
//
// The element tangent has more structure than beam_tail uses.  Rows 6..8 of
// the local stiffness are the negatives of rows 0..2 and f_cr[6..8] = -f_cr[0..2],
// so the unsymmetrised block rows are
//   [G0 H0 -G0 J0; G1 H1 -G1 J1; -G0 -H0 G0 -J0; G3 H3 -G3 J3],
// and the symmetrised tangent Ks_IJ = (X_IJ + X_JI^T) / 2 is fixed by six 3x3
// blocks:
//   S00 = sym(G0), S01 = (H0 + G1^T)/2, S11 = sym(H1),
//   S03 = (J0 + G3^T)/2, S13 = (J1 + H3^T)/2, S33 = sym(J3),
//   aa = [S00 S01; S01^T S11],  ab = [-S00 S03; -S01^T S13],  bb = [S00 -S03; -S03^T S33].
// Each local-stiffness row has at most two nonzeros against the rotation
// columns, so row r of A_I (the material part before the rotation to global
// axes) is a scaled row of P1 plus one of P2 (or of Q1, Q2), and Rcr^T A_I is
// the sum of the outer products R_r (x) A_I[r] over its nonzero rows, R_r the
// rows of Rcr.  The geometric term Rcr^T [f_I]x dpsi equals
// [g_I]x [e_x]x / L = (e_x g_I^T - (g_I . e_x) I) / L with g_I = Rcr^T f_I, the
// element's global force of block I.
// An element's outputs, 54 floats in shared memory (one slot per thread):
constexpr int EL_S00 = 0, EL_S11 = 6, EL_S33 = 12;   // symmetric: (0,0) (0,1) (0,2) (1,1) (1,2) (2,2)
constexpr int EL_S01 = 18, EL_S03 = 27, EL_S13 = 36;  // row-major
constexpr int EL_G0 = 45, EL_G1 = 48, EL_G3 = 51;     // f rows: node a translation g0, rotation g1; node b -g0, g3
constexpr int EL_BLK = 54;                            // the element's block ids aa, ab, ba, bb (int bits)
constexpr int EL_STRIDE = 59;  // odd: the threads' slots fall in different banks

XK_D int sym_index(int r, int c) {  // position of (r, c) in a symmetric 3x3 stored as 6 values
  const int i = r < c ? r : c, j = r < c ? c : r;
  return i == 0 ? j : (i == 1 ? 2 + j : 5);
}

// sym(X) of a row-major 3x3 into the 6-value form
XK_D void sym6(const float* X, float* S) {
  S[0] = X[0];
  S[1] = 0.5f * (X[1] + X[3]);
  S[2] = 0.5f * (X[2] + X[6]);
  S[3] = X[4];
  S[4] = 0.5f * (X[5] + X[7]);
  S[5] = X[8];
}

// M = sum of the outer products R_k (x) V_k (row-major)
XK_D void outer2(const float* Ra, const float* Va, const float* Rb, const float* Vb, float* M) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int c = 0; c < 3; ++c) M[3 * i + c] = Ra[i] * Va[c] + Rb[i] * Vb[c];
}
XK_D void outer3(const float* Ra, const float* Va, const float* Rb, const float* Vb, const float* Rc,
                 const float* Vc, float* M) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int c = 0; c < 3; ++c) M[3 * i + c] = Ra[i] * Va[c] + Rb[i] * Vb[c] + Rc[i] * Vc[c];
}

// One element: frame (the rotation vectors of both nodes by one thread), global forces of the
// blocks and, with want_K, the six symmetrised tangent blocks, written to the element's slot o
// (shared memory) as they are formed, so that few of them are held in registers at once.
// E: element record, NA / NB: the displacement part of the node records (u, 6 floats).
XK_D void beam_elem32(const float* __restrict__ E, const float* __restrict__ NA, const float* __restrict__ NB,
                      const xk_section& sec, bool want_K, float* o) {
  // the record as four 16-byte loads (64-byte aligned), the nodes' u as three 8-byte loads each
  const float4* E4 = reinterpret_cast<const float4*>(E);
  const float4 e0 = __ldg(E4), e1 = __ldg(E4 + 1), e2 = __ldg(E4 + 2), e3 = __ldg(E4 + 3);
  const float dx0[3] = {e0.x, e0.y, e0.z};
  const float L0 = e0.w;
  const float R0[9] = {e1.x, e1.y, e1.z, e1.w, e2.x, e2.y, e2.z, e2.w, e3.x};
  float ua[6], ub[6];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float2 pa = __ldg(reinterpret_cast<const float2*>(NA) + i), pb = __ldg(reinterpret_cast<const float2*>(NB) + i);
    ua[2 * i] = pa.x; ua[2 * i + 1] = pa.y;
    ub[2 * i] = pb.x; ub[2 * i + 1] = pb.y;
  }
  const float du[3] = {ub[0] - ua[0], ub[1] - ua[1], ub[2] - ua[2]};
  const float dxd[3] = {dx0[0] + du[0], dx0[1] + du[1], dx0[2] + du[2]};
  const float Ld = sqrtf(dot3(dxd, dxd));
  const float iLd = 1.0f / Ld;
  const float two_dx_du[3] = {2.0f * dx0[0] + du[0], 2.0f * dx0[1] + du[1], 2.0f * dx0[2] + du[2]};
  const float dax = dot3(du, two_dx_du) / (Ld + L0);
  const float ex[3] = {dxd[0] * iLd, dxd[1] * iLd, dxd[2] * iLd};
  float qr[4];
  {
    float v[3];
    cross3(R0, du, v);
    const float opc = fmaxf((Ld + L0 + dot3(R0, du)) * iLd, 1e-12f);
    const float w = sqrtf(0.5f * opc);
    const float kk = 0.5f * iLd / w;
    qr[0] = w; qr[1] = kk * v[0]; qr[2] = kk * v[1]; qr[3] = kk * v[2];
  }
  const float qrc[4] = {qr[0], -qr[1], -qr[2], -qr[3]};
  // local rotations theta_1, theta_2 = R0 log(q_rod^* (x) q_node)
  float t1[3], t2[3];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    float qn[4], qx[4], tx[3];
    quat_of_rotvecf(side ? ub + 3 : ua + 3, qn);
    qmulf(qrc, qn, qx);
    rotvec_of_quatf(qx, tx);
    float* t = side ? t2 : t1;
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = R0[3 * i] * tx[0] + R0[3 * i + 1] * tx[1] + R0[3 * i + 2] * tx[2];
  }
  float Rcr[9];
  {
    const float w = qr[0], x = qr[1], y = qr[2], z = qr[3];
    float Rrod[9];
    Rrod[0] = 1.f - 2.f * (y * y + z * z); Rrod[1] = 2.f * (x * y - w * z); Rrod[2] = 2.f * (x * z + w * y);
    Rrod[3] = 2.f * (x * y + w * z); Rrod[4] = 1.f - 2.f * (x * x + z * z); Rrod[5] = 2.f * (y * z - w * x);
    Rrod[6] = 2.f * (x * z - w * y); Rrod[7] = 2.f * (y * z + w * x); Rrod[8] = 1.f - 2.f * (x * x + y * y);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        Rcr[3 * i + j] = R0[3 * i] * Rrod[3 * j] + R0[3 * i + 1] * Rrod[3 * j + 1] + R0[3 * i + 2] * Rrod[3 * j + 2];
  }
  const KeCoef<float> kc = ke_coef<float>(sec, L0);
  // local forces of blocks 0, 1, 3 (block 2 = -block 0) and their global images g_I = Rcr^T f_I
  float g0[3], g1[3], g3[3];
  {
    const float f0[3] = {-kc.ea * dax, kc.k2z * (t1[2] + t2[2]), -kc.k2y * (t1[1] + t2[1])};
    const float f1[3] = {kc.gj * (t1[0] - t2[0]), kc.k1ay * t1[1] + kc.k1by * t2[1],
                         kc.k1az * t1[2] + kc.k1bz * t2[2]};
    const float f3[3] = {-f1[0], kc.k1by * t1[1] + kc.k1ay * t2[1], kc.k1bz * t1[2] + kc.k1az * t2[2]};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      g0[i] = Rcr[i] * f0[0] + Rcr[3 + i] * f0[1] + Rcr[6 + i] * f0[2];
      g1[i] = Rcr[i] * f1[0] + Rcr[3 + i] * f1[1] + Rcr[6 + i] * f1[2];
      g3[i] = Rcr[i] * f3[0] + Rcr[3 + i] * f3[1] + Rcr[6 + i] * f3[2];
      o[EL_G0 + i] = g0[i];
      o[EL_G1 + i] = g1[i];
      o[EL_G3 + i] = g3[i];
    }
  }
  if (!want_K) return;
  const float* R_0 = Rcr;
  const float* R_1 = Rcr + 3;
  const float* R_2 = Rcr + 6;
  // P_s = T^-1(t_s) dpsi with dpsi = Rcr [e_x]x / L: row i of M [e_x]x is M_i x e_x, M = T^-1 Rcr;
  // Q_s = T^-1(t_s) Rcr T(theta_node)
  float P1[9], P2[9], Q1[9], Q2[9];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    float Ti[9], Ts[9], M[9];
    tangent_ops<float>(side ? t2 : t1, true, Ti);
    tangent_ops<float>(side ? ub + 3 : ua + 3, false, Ts);
    mm3(Ti, Rcr, M);
    float* P = side ? P2 : P1;
    float* Q = side ? Q2 : Q1;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      float c[3];
      cross3(M + 3 * i, ex, c);
      P[3 * i] = c[0] * iLd;
      P[3 * i + 1] = c[1] * iLd;
      P[3 * i + 2] = c[2] * iLd;
    }
    mm3(M, Ts, Q);
  }
  // G_I = Rcr^T A_I + geometric term; G1^T / 2 and G3^T / 2 go to the S01 and S03 slots at once
  // (0.5 x + 0.5 y rounds as 0.5 (x + y)), so that P1, P2 and the forces end here
  {
    float v0[3], v1[3], v2[3], G[9];
    const float d1 = dot3(g1, ex), d3 = dot3(g3, ex), d0 = dot3(g0, ex);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v0[c] = kc.gj * (P1[c] - P2[c]);
      v1[c] = kc.k1ay * P1[3 + c] + kc.k1by * P2[3 + c];
      v2[c] = kc.k1az * P1[6 + c] + kc.k1bz * P2[6 + c];
    }
    outer3(R_0, v0, R_1, v1, R_2, v2, G);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        o[EL_S01 + 3 * c + i] = 0.5f * (G[3 * i + c] + iLd * (ex[i] * g1[c] - (i == c ? d1 : 0.f)));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v0[c] = -v0[c];
      v1[c] = kc.k1by * P1[3 + c] + kc.k1ay * P2[3 + c];
      v2[c] = kc.k1bz * P1[6 + c] + kc.k1az * P2[6 + c];
    }
    outer3(R_0, v0, R_1, v1, R_2, v2, G);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        o[EL_S03 + 3 * c + i] = 0.5f * (G[3 * i + c] + iLd * (ex[i] * g3[c] - (i == c ? d3 : 0.f)));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v0[c] = kc.ea * ex[c];
      v1[c] = kc.k2z * (P1[6 + c] + P2[6 + c]);
      v2[c] = -kc.k2y * (P1[3 + c] + P2[3 + c]);
    }
    outer3(R_0, v0, R_1, v1, R_2, v2, G);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int c = 0; c < 3; ++c) G[3 * i + c] += iLd * (ex[i] * g0[c] - (i == c ? d0 : 0.f));
    float S[6];
    sym6(G, S);
#pragma unroll
    for (int i = 0; i < 6; ++i) o[EL_S00 + i] = S[i];
  }
  {
    float a1[3], a2[3], b0[3], X[9], S[6];
    // H0, J0: the I = 0 rows against Q1, Q2, added to the halves of G1^T, G3^T
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      a1[c] = kc.k2z * Q1[6 + c];
      a2[c] = -kc.k2y * Q1[3 + c];
    }
    outer2(R_1, a1, R_2, a2, X);
#pragma unroll
    for (int i = 0; i < 9; ++i) o[EL_S01 + i] += 0.5f * X[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      a1[c] = kc.k2z * Q2[6 + c];
      a2[c] = -kc.k2y * Q2[3 + c];
    }
    outer2(R_1, a1, R_2, a2, X);
#pragma unroll
    for (int i = 0; i < 9; ++i) o[EL_S03 + i] += 0.5f * X[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      b0[c] = kc.gj * Q1[c];
      a1[c] = kc.k1ay * Q1[3 + c];
      a2[c] = kc.k1az * Q1[6 + c];
    }
    outer3(R_0, b0, R_1, a1, R_2, a2, X);  // H1
    sym6(X, S);
#pragma unroll
    for (int i = 0; i < 6; ++i) o[EL_S11 + i] = S[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      b0[c] = kc.gj * Q2[c];
      a1[c] = kc.k1ay * Q2[3 + c];
      a2[c] = kc.k1az * Q2[6 + c];
    }
    outer3(R_0, b0, R_1, a1, R_2, a2, X);  // J3
    sym6(X, S);
#pragma unroll
    for (int i = 0; i < 6; ++i) o[EL_S33 + i] = S[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      b0[c] = -kc.gj * Q1[c];
      a1[c] = kc.k1by * Q1[3 + c];
      a2[c] = kc.k1bz * Q1[6 + c];
    }
    outer3(R_0, b0, R_1, a1, R_2, a2, X);  // H3
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int c = 0; c < 3; ++c) o[EL_S13 + 3 * c + i] = 0.5f * X[3 * i + c];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      b0[c] = -kc.gj * Q2[c];
      a1[c] = kc.k1by * Q2[3 + c];
      a2[c] = kc.k1bz * Q2[6 + c];
    }
    outer3(R_0, b0, R_1, a1, R_2, a2, X);  // J1
#pragma unroll
    for (int i = 0; i < 9; ++i) o[EL_S13 + i] += 0.5f * X[i];
  }
}

// Value (r, c) of a stored 6x6 block of one element, from its slot o:
// aa = [S00 S01; S01^T S11], bb = [S00 -S03; -S03^T S33], ab = [-S00 S03; -S01^T S13] (rows: node a).
XK_D float blk_aa(const float* o, int r, int c) {
  if (r < 3) return c < 3 ? o[EL_S00 + sym_index(r, c)] : o[EL_S01 + 3 * r + c - 3];
  return c < 3 ? o[EL_S01 + 3 * c + r - 3] : o[EL_S11 + sym_index(r - 3, c - 3)];
}
XK_D float blk_bb(const float* o, int r, int c) {
  if (r < 3) return c < 3 ? o[EL_S00 + sym_index(r, c)] : -o[EL_S03 + 3 * r + c - 3];
  return c < 3 ? -o[EL_S03 + 3 * c + r - 3] : o[EL_S33 + sym_index(r - 3, c - 3)];
}
XK_D float blk_ab(const float* o, int r, int c) {
  if (r < 3) return c < 3 ? -o[EL_S00 + sym_index(r, c)] : o[EL_S03 + 3 * r + c - 3];
  return c < 3 ? -o[EL_S01 + 3 * c + r - 3] : o[EL_S13 + 3 * (r - 3) + c - 3];
}

// block kinds of an element: 0 aa, 1 ab, 2 ba (the transpose of ab), 3 bb; 4: aa of o plus bb of p
XK_D float blk_val(int kind, const float* o, const float* p, int r, int c) {
  switch (kind) {
    case 0: return blk_aa(o, r, c);
    case 1: return blk_ab(o, r, c);
    case 2: return blk_ab(o, c, r);
    case 3: return blk_bb(o, r, c);
    default: return blk_aa(o, r, c) + blk_bb(p, r, c);
  }
}

// HOW: 0 store, 1 add to the stored value, 2 atomic add
template <int KIND, int HOW>
XK_D void put_block(float* __restrict__ dst, const float* o, const float* p) {
  float4* d = reinterpret_cast<float4*>(dst);
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    float v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = blk_val(KIND, o, p, (4 * q + k) / 6, (4 * q + k) % 6);
    float4 x = make_float4(v[0], v[1], v[2], v[3]);
    if (HOW == 2) {
      atomicAdd(d + q, x);
    } else {
      if (HOW == 1) {
        const float4 y = d[q];
        x.x += y.x; x.y += y.y; x.z += y.z; x.w += y.w;
      }
      d[q] = x;
    }
  }
}

// f rows of one node: translation t (3, negated with neg_t) then rotation r (3), as doubles
template <int HOW>  // 0 store, 1 add, 2 atomic add
XK_D void put_rows(double* __restrict__ f, long long node, const float* t, const float* r, bool neg_t) {
  double v[6];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    v[i] = xk_f2d(neg_t ? -t[i] : t[i]);
    v[3 + i] = xk_f2d(r[i]);
  }
  double* d = f + 6 * node;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    if (HOW == 0) d[i] = v[i];
    else if (HOW == 1) d[i] += v[i];
    else atomicAdd(d + i, v[i]);
  }
}

// The float CR beam, one thread per element, its outputs staged in a shared-memory slot.
//
// BEAM_ORDERED (wire meshes whose elements follow each other along every wire:
// element e's node b is element e+1's node a, or the node has one element):
// a warp covers 31 elements; lane j takes element 31 w + j - 1, and lane 0's
// element (the last of the previous warp) is computed only for its node-b
// block and rows.  Lane j writes the diagonal block and f rows of its node a
// as its own block aa plus lane j-1's block bb (read from that lane's slot),
// so every stored block and f row has one writer and no zeroing pass is
// needed; the sum a + b equals the other modes' 0 + a + b and their
// store-then-add bits.  A lane whose predecessor ends its wire (or the mesh)
// writes the predecessor's bb and node-b rows instead.
// BEAM_ATOMIC (other chain meshes): node rows and diagonal blocks zeroed
// first (k_beam_zero32), the two contributions of a shared node added by
// atomics.  BEAM_COLOUR: elements of one colour of the plan, the first writer
// of a block stores and later colours add.
// The mode is a launch argument, not a template parameter: the element's arithmetic is compiled
// once, so that every mode computes the same bits for an element (with floating-point contraction
// left to the compiler, separately compiled copies may round differently).
// Six CTAs of 128 threads per SM (80 registers, 30 KB of slots each): 152 SMs hold 3,648 warps, i.e.
// up to 113k ordered elements in one wave, without a second round of the long per-thread chain.
constexpr int BEAMW_T = 128;
constexpr int BEAM_ORDERED = 0, BEAM_ATOMIC = 1, BEAM_COLOUR = 2;

// One element of the launch (t: the thread's logical index), its outputs staged in the slots.
XK_D void beam_item(int mode, long long t, const xk_mesh& m, const xk_section& sec, const float* __restrict__ e32,
                    const int32_t* __restrict__ order, int k0, int k1, const int32_t* __restrict__ blk,
                    const uint8_t* __restrict__ first, const float* __restrict__ n32, double* __restrict__ f_int,
                    float* __restrict__ Kv, float* slots) {
  const int lane = threadIdx.x & 31;
  const long long ne = m.n_elems;
  long long e;
  bool live;
  if (mode == BEAM_ORDERED) {
    e = 31 * (t >> 5) + lane - 1;
    live = e >= 0 && e < ne;
  } else {
    const long long k = k0 + t;
    live = k < k1;
    if (!live) return;  // no exchange between threads in these modes
    e = mode == BEAM_COLOUR ? order[k] : k;
  }
  const bool want_K = Kv != nullptr;
  float* o = slots + threadIdx.x * EL_STRIDE;
  int a = -1, b = -1;
  int* ob = reinterpret_cast<int*>(o + EL_BLK);
  if (live) {
    // the block ids are loaded with the connectivity, before the element's chain, and parked in the slot
    const int2 ab = __ldg(reinterpret_cast<const int2*>(m.conn) + e);
    if (want_K) {
      const int4 bi = __ldg(reinterpret_cast<const int4*>(blk) + e);
      ob[0] = bi.x; ob[1] = bi.y; ob[2] = bi.z; ob[3] = bi.w;
    }
    a = ab.x;
    b = ab.y;
    beam_elem32(e32 + e * XK_ELEM32_STRIDE, n32 + (long long)a * XK_NODE32_STRIDE + 6,
                n32 + (long long)b * XK_NODE32_STRIDE + 6, sec, want_K, o);
  }
  if (mode == BEAM_ORDERED) {
    const int bp = __shfl_up_sync(0xffffffffu, b, 1);  // the predecessor's node b
    __syncwarp();
    if (lane == 0 || e > ne) return;
    const float* p = o - EL_STRIDE;          // the predecessor's slot
    const bool pred = e >= 1;                // the predecessor exists (e <= ne here)
    const bool joined = live && pred && bp == a;
    if (pred && !joined) {                   // the predecessor ends its wire: its node b alone
      if (f_int) put_rows<0>(f_int, bp, p + EL_G0, p + EL_G3, true);
      if (want_K) put_block<3, 0>(Kv + 36LL * reinterpret_cast<const int*>(p + EL_BLK)[3], p, p);
    }
    if (!live) return;
    if (f_int) {
      double v[6];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        v[i] = xk_f2d(o[EL_G0 + i]);
        v[3 + i] = xk_f2d(o[EL_G1 + i]);
        if (joined) {
          v[i] += xk_f2d(-p[EL_G0 + i]);
          v[3 + i] += xk_f2d(p[EL_G3 + i]);
        }
      }
      if (((uintptr_t)f_int & 15) == 0) {
        double2* d = reinterpret_cast<double2*>(f_int + 6LL * a);
#pragma unroll
        for (int i = 0; i < 3; ++i) d[i] = make_double2(v[2 * i], v[2 * i + 1]);
      } else {
#pragma unroll
        for (int i = 0; i < 6; ++i) f_int[6LL * a + i] = v[i];
      }
    }
    if (!want_K) return;
    if (joined) put_block<4, 0>(Kv + 36LL * ob[0], o, p);
    else put_block<0, 0>(Kv + 36LL * ob[0], o, o);
    if (ob[1] >= 0) put_block<1, 0>(Kv + 36LL * ob[1], o, o);
    else put_block<2, 0>(Kv + 36LL * ob[2], o, o);
    return;
  }
  const uint8_t fl = mode == BEAM_COLOUR ? first[e] : 0;
  if (f_int) {
    if (mode == BEAM_ATOMIC) {
      put_rows<2>(f_int, a, o + EL_G0, o + EL_G1, false);
      put_rows<2>(f_int, b, o + EL_G0, o + EL_G3, true);
    } else {
      if (fl & 1) put_rows<0>(f_int, a, o + EL_G0, o + EL_G1, false);
      else put_rows<1>(f_int, a, o + EL_G0, o + EL_G1, false);
      if (fl & 8) put_rows<0>(f_int, b, o + EL_G0, o + EL_G3, true);
      else put_rows<1>(f_int, b, o + EL_G0, o + EL_G3, true);
    }
  }
  if (!want_K) return;
  if (mode == BEAM_ATOMIC) {
    put_block<0, 2>(Kv + 36LL * ob[0], o, o);
    put_block<3, 2>(Kv + 36LL * ob[3], o, o);
  } else {
    if (fl & 1) put_block<0, 0>(Kv + 36LL * ob[0], o, o);
    else put_block<0, 1>(Kv + 36LL * ob[0], o, o);
    if (fl & 8) put_block<3, 0>(Kv + 36LL * ob[3], o, o);
    else put_block<3, 1>(Kv + 36LL * ob[3], o, o);
  }
  // the off-diagonal block has one writer
  if (ob[1] >= 0) put_block<1, 0>(Kv + 36LL * ob[1], o, o);
  else put_block<2, 0>(Kv + 36LL * ob[2], o, o);
}

// Launch: the logical threads of the mode (32 per warp of 31 ordered elements, or one per element of
// the colour range), each CTA thread taking every (gridDim.x * BEAMW_T)-th; a full grid gives one
// element to each thread, a smaller one (the plan's beam_ctas_per_sm) loops, so that the beam can
// run beside the bandwidth-bound pair kernels on few SMs' worth of warps.  A warp's slots are rewritten
// only after all of its lanes have finished reading them.
__global__ void __launch_bounds__(BEAMW_T, 6) k_beam32e(int mode, xk_mesh m, xk_section sec,
                                                     const float* __restrict__ e32,
                                                     const int32_t* __restrict__ order, int k0, int k1,
                                                     const int32_t* __restrict__ blk,
                                                     const uint8_t* __restrict__ first,
                                                     const float* __restrict__ n32, double* __restrict__ f_int,
                                                     float* __restrict__ Kv, long long n_threads) {
  __shared__ float slots[BEAMW_T * EL_STRIDE];
  const long long stride = (long long)gridDim.x * BEAMW_T;  // a multiple of 32
  for (long long t = (long long)blockIdx.x * BEAMW_T + threadIdx.x; t < n_threads; t += stride) {
    if (mode == BEAM_ORDERED) __syncwarp();  // the whole warp is here: n_threads is a multiple of 32 there
    beam_item(mode, t, m, sec, e32, order, k0, k1, blk, first, n32, f_int, Kv, slots);
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

// CTAs of a float beam launch over `threads` logical threads: one per thread, or at most
// plan->beam_ctas_per_sm per SM (the kernel loops)
static int beam_grid(long long threads, const xk_beam_plan* plan) {
  const int full = xk_blocks(threads, BEAMW_T);
  if (plan->beam_ctas_per_sm <= 0) return full;
  const long long cap = (long long)plan->beam_ctas_per_sm * xk_sm_count();
  return full < cap ? full : (int)cap;
}

extern "C" xk_status xk_beam_assemble32(const xk_mesh* m, const xk_section* sec, const float* elem32,
                                        const xk_beam_plan* plan, const float* node32, double* f_int, float* K_vals,
                                        xk_stream s) {
  if (!m || !sec || !elem32 || !plan || !node32) return xk_set_error(XK_ERR_ARG, "xk_beam_assemble32: null argument");
  if (((uintptr_t)elem32 & 15) || ((uintptr_t)node32 & 7) || ((uintptr_t)m->conn & 7) || ((uintptr_t)plan->blk & 15))
    return xk_set_error(XK_ERR_ARG, "xk_beam_assemble32: elem32 and the plan's blk must be 16-byte aligned, node32 "
                                    "and conn 8-byte aligned");
  if (!f_int && !K_vals) return XK_OK;
  cudaStream_t st = (cudaStream_t)s;
  if (plan->node_diag) {  // chain mesh: one launch over all elements
    const long long ne = m->n_elems;
    if (ne == 0) return XK_OK;
    if (plan->chain_ordered) {  // 31 elements per warp, the lane before them repeating the previous one
      const long long threads = 32 * (ne / 31 + 1);
      k_beam32e<<<beam_grid(threads, plan), BEAMW_T, 0, st>>>(BEAM_ORDERED, *m, *sec, elem32, nullptr, 0, 0, plan->blk,
                                                             plan->first, node32, f_int, K_vals, threads);
    } else {
      k_beam_zero32<<<xk_blocks(9LL * m->n_nodes, 256), 256, 0, st>>>(m->n_nodes, plan->node_diag, f_int, K_vals);
      k_beam32e<<<beam_grid(ne, plan), BEAMW_T, 0, st>>>(BEAM_ATOMIC, *m, *sec, elem32, nullptr, 0, (int)ne, plan->blk,
                                                         plan->first, node32, f_int, K_vals, ne);
    }
    XK_CHECK_LAUNCH();
    return XK_OK;
  }
  for (int c = 0; c < plan->n_colors; ++c) {
    const int k0 = plan->color_ptr_host[c], k1 = plan->color_ptr_host[c + 1];
    if (k1 <= k0) continue;
    k_beam32e<<<beam_grid(k1 - k0, plan), BEAMW_T, 0, st>>>(BEAM_COLOUR, *m, *sec, elem32, plan->elem_order, k0, k1,
                                                           plan->blk, plan->first, node32, f_int, K_vals, k1 - k0);
    XK_CHECK_LAUNCH();
  }
  return XK_OK;
}
