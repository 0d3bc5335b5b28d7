// Segment-segment closest point in exact reference arithmetic, shared by the pair kernels and the
// pruning features.
#pragma once

#include "xk_common.cuh"

// _closest_point_segments_batch (geometry/_compute.py:55-151), operation for operation.
XK_D void closest_exact(const double* xA0, const double* xA1, const double* xB0, const double* xB1, double& s,
                        double& t, double& dist, double* normal, double* diff) {
  const double TOL = 1e-10;
  double dA[3], dB[3], w0[3];
  for (int i = 0; i < 3; ++i) {
    dA[i] = xsub(xA1[i], xA0[i]);
    dB[i] = xsub(xB1[i], xB0[i]);
    w0[i] = xsub(xA0[i], xB0[i]);
  }
  const double a = xdot_es(dA, dA), b = xdot_es(dA, dB), c = xdot_es(dB, dB);
  const double d = xdot_es(dA, w0), e = xdot_es(dB, w0);
  const double det = xsub(xmul(a, c), xmul(b, b));
  double ac = xmul(a, c);
  if (!(ac >= 1e-30)) ac = (ac != ac) ? ac : 1e-30;  // np.maximum keeps NaN
  const bool par = det < xmul(TOL, ac);
  const double sdet = par ? 1.0 : det;
  const double s_unc = par ? 0.0 : xdiv(xsub(xmul(b, e), xmul(c, d)), sdet);
  const double t_unc = par ? 0.0 : xdiv(xsub(xmul(a, e), xmul(b, d)), sdet);
  const bool cok = c > TOL, aok = a > TOL;
  const double sc = cok ? c : 1.0, sa = aok ? a : 1.0;
  s = par ? 0.0 : xclip01(s_unc);
  t = par ? (cok ? xclip01(xdiv(e, sc)) : 0.0) : xclip01(t_unc);
  const bool s_cl = (s_unc < 0.0) || (s_unc > 1.0);
  const bool t_cl = (t_unc < 0.0) || (t_unc > 1.0);
  if (s_cl && !par) t = cok ? xclip01(xdiv(xadd(xmul(b, s), e), sc)) : 0.0;
  if (t_cl && !par) {
    s = aok ? xclip01(xdiv(xsub(xmul(b, t), d), sa)) : 0.0;
    t = cok ? xclip01(xdiv(xadd(xmul(b, s), e), sc)) : 0.0;
  }
  for (int i = 0; i < 3; ++i) diff[i] = xsub(xadd(xA0[i], xmul(s, dA[i])), xadd(xB0[i], xmul(t, dB[i])));
  dist = xsqrt(xdot_es(diff, diff));
  const double sd = (dist >= 1e-30 || dist != dist) ? dist : 1e-30;
  for (int i = 0; i < 3; ++i) normal[i] = xdiv(diff[i], sd);
  if (dist < 1e-30) { normal[0] = 0.0; normal[1] = 0.0; normal[2] = 1.0; }
}

