// Contact pairs: narrowphase, Huber normal force, Coulomb return mapping and
// the factorised pair tangent.  One thread per pair; contributing pairs and
// the rest run as two launches over the per-increment lists so that warps do
// not diverge between the two kinds of work.
#include <cuda.h>

#include <atomic>
#include <cmath>
#include <mutex>

#include "xk_common.cuh"
#include "segment.cuh"

namespace {

constexpr int PAIR_T = 256;
constexpr uint8_t ST_INACTIVE = 0, ST_ACTIVE = 1, ST_SLIDING = 2;

struct PairNodes {
  int n[4];
};

XK_D PairNodes pair_nodes(const xk_mesh& m, int ea, int eb) {
  PairNodes p;
  p.n[0] = m.conn[2 * ea];
  p.n[1] = m.conn[2 * ea + 1];
  p.n[2] = m.conn[2 * eb];
  p.n[3] = m.conn[2 * eb + 1];
  return p;
}

// Deformed coordinates X + u[0:3] (DeformedCoordsProcess, contact/solver/_utils.py:16-28).
XK_D void deformed(const xk_mesh& m, const double* u, int node, double* x) {
  x[0] = xadd(m.X[3LL * node], u[6LL * node]);
  x[1] = xadd(m.X[3LL * node + 1], u[6LL * node + 1]);
  x[2] = xadd(m.X[3LL * node + 2], u[6LL * node + 2]);
}

// _build_contact_frame_batch (geometry/_compute.py:154-261) for one pair, reference op order.
XK_D void frame_exact(const double* nrm, const double* pt1, const double* pn, double* n, double* t1, double* t2) {
  double nn = xsqrt(xdot_es(nrm, nrm));
  if (!(nn >= 1e-30)) nn = (nn != nn) ? nn : 1e-30;
  for (int i = 0; i < 3; ++i) n[i] = xdiv(nrm[i], nn);
  const bool has_t1 = xsqrt(xdot_es(pt1, pt1)) > 1e-10;
  const double pnn = xsqrt(xdot_es(pn, pn));
  const bool has_n = pnn > 1e-10;
  bool done = false;
  if (has_t1 && has_n) {
    double so = (pnn >= 1e-30) ? pnn : 1e-30;
    double no[3] = {xdiv(pn[0], so), xdiv(pn[1], so), xdiv(pn[2], so)};
    double v[3];
    xcross(no, n, v);
    const double sv = xsqrt(xdot_es(v, v));
    const double cv = xdot_es(no, n);
    double tr[3] = {pt1[0], pt1[1], pt1[2]};
    if (sv >= 1e-12) {
      double vx[3], vvx[3];
      xcross(v, pt1, vx);
      xcross(v, vx, vvx);
      const double f = xdiv(xsub(1.0, cv), xmul(sv, sv));
      for (int i = 0; i < 3; ++i) tr[i] = xadd(xadd(pt1[i], vx[i]), xmul(f, vvx[i]));
    }
    const double dn = xdot_es(tr, n);
    double raw[3];
    for (int i = 0; i < 3; ++i) raw[i] = xsub(tr[i], xmul(dn, n[i]));
    const double nr = xsqrt(xdot_es(raw, raw));
    if (nr > 1e-10) {
      for (int i = 0; i < 3; ++i) t1[i] = xdiv(raw[i], nr);
      xcross(n, t1, t2);
      done = true;
    }
  }
  if (!done && has_t1) {
    const double dn = xdot_es(pt1, n);
    double raw[3];
    for (int i = 0; i < 3; ++i) raw[i] = xsub(pt1[i], xmul(dn, n[i]));
    const double nr = xsqrt(xdot_es(raw, raw));
    if (nr > 1e-10) {
      for (int i = 0; i < 3; ++i) t1[i] = xdiv(raw[i], nr);
      xcross(n, t1, t2);
      done = true;
    }
  }
  if (!done) {
    double ref[3] = {0.0, 0.0, 0.0};
    const double a0 = fabs(n[0]), a1 = fabs(n[1]), a2 = fabs(n[2]);
    ref[(a0 <= a1 && a0 <= a2) ? 0 : (a1 <= a2 ? 1 : 2)] = 1.0;
    const double dn = xdot_es(ref, n);
    double raw[3];
    for (int i = 0; i < 3; ++i) raw[i] = xsub(ref[i], xmul(dn, n[i]));
    double nr = xsqrt(xdot_es(raw, raw));
    if (!(nr >= 1e-30)) nr = (nr != nr) ? nr : 1e-30;
    for (int i = 0; i < 3; ++i) t1[i] = xdiv(raw[i], nr);
    xcross(n, t1, t2);
  }
}

// Mixed-precision closest point: the difference vectors and the distance are
// double, the 2x2 parameter solve is float unless the segments are close to
// parallel, in which case the exact routine decides.
XK_D void closest_mixed(const double* xA0, const double* xA1, const double* xB0, const double* xB1, double& s,
                        double& t, double& dist, double* normal) {
  double dA[3], dB[3], w0[3];
  for (int i = 0; i < 3; ++i) {
    dA[i] = xA1[i] - xA0[i];
    dB[i] = xB1[i] - xB0[i];
    w0[i] = xA0[i] - xB0[i];
  }
  float fa[3] = {(float)dA[0], (float)dA[1], (float)dA[2]};
  float fb[3] = {(float)dB[0], (float)dB[1], (float)dB[2]};
  float fw[3] = {(float)w0[0], (float)w0[1], (float)w0[2]};
  float a = dot3(fa, fa), b = dot3(fa, fb), c = dot3(fb, fb), d = dot3(fa, fw), e = dot3(fb, fw);
  float ac = a * c;
  float det = ac - b * b;
  if (!(det > 1e-3f * ac)) {  // near-parallel or degenerate: exact double routine
    double diff[3];
    closest_exact(xA0, xA1, xB0, xB1, s, t, dist, normal, diff);
    return;
  }
  float idet = 1.0f / det;
  float su = (b * e - c * d) * idet, tu = (a * e - b * d) * idet;
  float sf = fminf(fmaxf(su, 0.0f), 1.0f), tf = fminf(fmaxf(tu, 0.0f), 1.0f);
  if (su < 0.0f || su > 1.0f) tf = fminf(fmaxf((b * sf + e) / c, 0.0f), 1.0f);
  if (tu < 0.0f || tu > 1.0f) {
    sf = fminf(fmaxf((b * tf - d) / a, 0.0f), 1.0f);
    tf = fminf(fmaxf((b * sf + e) / c, 0.0f), 1.0f);
  }
  s = sf;
  t = tf;
  double diff[3];
  for (int i = 0; i < 3; ++i) diff[i] = w0[i] + s * dA[i] - t * dB[i];
  dist = sqrt(diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2]);
  if (dist < 1e-30) { normal[0] = 0.0; normal[1] = 0.0; normal[2] = 1.0; return; }
  const double id = 1.0 / dist;
  for (int i = 0; i < 3; ++i) normal[i] = diff[i] * id;
}

// Frame transport in float; (1-c)/s^2 is written 1/(1+c), equal for unit vectors.
XK_D void frame_mixed(const double* nrm, const double* pt1d, const double* pnd, double* nout, double* t1o,
                      double* t2o) {
  float n[3] = {(float)nrm[0], (float)nrm[1], (float)nrm[2]};
  float inv = rsqrtf(fmaxf(dot3(n, n), 1e-30f));
  for (int i = 0; i < 3; ++i) n[i] *= inv;
  float pt1[3] = {(float)pt1d[0], (float)pt1d[1], (float)pt1d[2]};
  float pn[3] = {(float)pnd[0], (float)pnd[1], (float)pnd[2]};
  const bool has_t1 = dot3(pt1, pt1) > 1e-20f, has_n = dot3(pn, pn) > 1e-20f;
  float t1[3], t2[3];
  bool done = false;
  if (has_t1) {
    float tr[3] = {pt1[0], pt1[1], pt1[2]};
    if (has_n) {
      float ip = rsqrtf(dot3(pn, pn));
      float no[3] = {pn[0] * ip, pn[1] * ip, pn[2] * ip};
      float v[3], vx[3], vvx[3];
      cross3(no, n, v);
      float cv = dot3(no, n);
      float s2 = dot3(v, v);
      // (1 - c) / s^2 of the reference equals 1 / (1 + c) for unit vectors and
      // has no cancellation; near c = -1 the reference form is the stable one
      if (cv > 0.0f || s2 >= 1e-24f) {
        cross3(v, pt1, vx);
        cross3(v, vx, vvx);
        float f = cv > 0.0f ? 1.0f / (1.0f + cv) : (1.0f - cv) / s2;
        for (int i = 0; i < 3; ++i) tr[i] = pt1[i] + vx[i] + f * vvx[i];
      }
    }
    float dn = dot3(tr, n);
    float raw[3] = {tr[0] - dn * n[0], tr[1] - dn * n[1], tr[2] - dn * n[2]};
    float r2 = dot3(raw, raw);
    if (r2 > 1e-20f) {
      float ir = rsqrtf(r2);
      for (int i = 0; i < 3; ++i) t1[i] = raw[i] * ir;
      done = true;
    }
  }
  if (!done) {
    float ref[3] = {0.f, 0.f, 0.f};
    float a0 = fabsf(n[0]), a1 = fabsf(n[1]), a2 = fabsf(n[2]);
    ref[(a0 <= a1 && a0 <= a2) ? 0 : (a1 <= a2 ? 1 : 2)] = 1.0f;
    float dn = dot3(ref, n);
    float raw[3] = {ref[0] - dn * n[0], ref[1] - dn * n[1], ref[2] - dn * n[2]};
    float ir = rsqrtf(fmaxf(dot3(raw, raw), 1e-30f));
    for (int i = 0; i < 3; ++i) t1[i] = raw[i] * ir;
  }
  cross3(n, t1, t2);
  for (int i = 0; i < 3; ++i) { nout[i] = n[i]; t1o[i] = t1[i]; t2o[i] = t2[i]; }
}

XK_D void load3(const double* base, long long stride, long long i, double* v) {
  v[0] = base[i];
  v[1] = base[stride + i];
  v[2] = base[2 * stride + i];
}
XK_D void store3(double* base, long long stride, long long i, const double* v) {
  base[i] = v[0];
  base[stride + i] = v[1];
  base[2 * stride + i] = v[2];
}

// Coated wires (_manager_process.py:351-360): coat_total = (r_a - core_a) + (r_b - core_b) and the
// compression max(0, coat_total - gap) of the core gap.
XK_D double coat_total_of(const xk_mesh& m, int ea, int eb) {
  return xadd(xsub(m.radii[ea], m.core_radii[ea]), xsub(m.radii[eb], m.core_radii[eb]));
}
XK_D double coat_compression(const xk_mesh& m, int ea, int eb, double gap) {
  return fmax(0.0, xsub(coat_total_of(m, ea, eb), gap));
}

XK_D void narrow_exact_one(const xk_mesh& m, xk_pairs& p, const double* __restrict__ u, double g_on, double g_off,
                           int allow_deact, int update_active, int i) {
  const long long cap = p.cap;
  PairNodes nd = pair_nodes(m, p.ea[i], p.eb[i]);
  double x[4][3];
  for (int k = 0; k < 4; ++k) deformed(m, u, nd.n[k], x[k]);
  double s, t, dist, nrm[3], diff[3];
  closest_exact(x[0], x[1], x[2], x[3], s, t, dist, nrm, diff);
  const bool coat = m.core_radii != nullptr;
  const double gap = coat ? xsub(dist, xadd(m.core_radii[p.ea[i]], m.core_radii[p.eb[i]]))
                          : xsub(dist, xadd(m.radii[p.ea[i]], m.radii[p.eb[i]]));
  const double cc = coat ? coat_compression(m, p.ea[i], p.eb[i], gap) : 0.0;
  if (coat && p.coat_cc) p.coat_cc[i] = cc;
  double pt1[3], pn[3], n[3], t1[3], t2[3];
  load3(p.t1, cap, i, pt1);
  load3(p.normal, cap, i, pn);
  frame_exact(nrm, pt1, pn, n, t1, t2);
  p.s[i] = s;
  p.t[i] = t;
  p.gap[i] = gap;
  store3(p.normal, cap, i, n);
  store3(p.t1, cap, i, t1);
  store3(p.t2, cap, i, t2);
  if (update_active) {  // _update_active_set_state (_manager_process.py:475-494), coating term included
    const bool coat_active = coat && cc > 0.0;
    uint8_t st = p.status[i];
    if (st == ST_INACTIVE) {
      if (gap <= g_on || coat_active) p.status[i] = ST_ACTIVE;
    } else if (allow_deact && gap >= g_off && !coat_active) {
      p.status[i] = ST_INACTIVE;
    }
  }
}

__global__ void k_narrow_exact(xk_mesh m, xk_pairs p, const double* __restrict__ u, double g_on, double g_off,
                               int allow_deact, int update_active) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < p.n) narrow_exact_one(m, p, u, g_on, g_off, allow_deact, update_active, i);
}

XK_HD double huber(double x, double d) {  // contact_force/strategy.py:104-113
  if (d <= 0.0) return x > 0.0 ? x : 0.0;
  if (x < -d) return 0.0;
  if (x > d) return x;
  return (x + d) * (x + d) / (4.0 * d);
}
XK_HD double huber_deriv(double x, double d) {  // contact_force/strategy.py:115-124
  if (d <= 0.0) return x > 0.0 ? 1.0 : 0.0;
  if (x < -d) return 0.0;
  if (x > d) return 1.0;
  return (x + d) / (2.0 * d);
}

// Narrowphase of one pair at X + u, exact (FP64) or mixed, written to the pair table.
template <int P>
XK_D void pair_narrow(const xk_mesh& m, xk_pairs& p, int i, const int* nd, const double* __restrict__ u, double& s,
                      double& t, double& gap, double* n, double* t1, double* t2) {
  const long long cap = p.cap;
  const bool coat = m.core_radii != nullptr;  // coated wires: the gap between the cores
  const double ra = coat ? m.core_radii[p.ea[i]] : m.radii[p.ea[i]];
  const double rb = coat ? m.core_radii[p.eb[i]] : m.radii[p.eb[i]];
  double x[4][3];
  for (int k = 0; k < 4; ++k)
    for (int c = 0; c < 3; ++c) x[k][c] = xadd(m.X[3LL * nd[k] + c], u[6LL * nd[k] + c]);
  double dist, nrm[3], pt1[3], pn[3];
  load3(p.t1, cap, i, pt1);
  load3(p.normal, cap, i, pn);
  if (P == XK_FP64) {
    double diff[3];
    closest_exact(x[0], x[1], x[2], x[3], s, t, dist, nrm, diff);
    gap = xsub(dist, xadd(ra, rb));
    frame_exact(nrm, pt1, pn, n, t1, t2);
  } else {
    closest_mixed(x[0], x[1], x[2], x[3], s, t, dist, nrm);
    gap = dist - (ra + rb);
    frame_mixed(nrm, pt1, pn, n, t1, t2);
  }
  p.s[i] = s;
  p.t[i] = t;
  p.gap[i] = gap;
  store3(p.normal, cap, i, n);
  store3(p.t1, cap, i, t1);
  store3(p.t2, cap, i, t2);
  if (coat && p.coat_cc) p.coat_cc[i] = coat_compression(m, p.ea[i], p.eb[i], gap);
}

// Kelvin-Voigt coating of one pair (KelvinVoigtCoatingProcess, contact/coating/strategy.py:97-370) as
// additions to its combined record: the spring / dashpot force v = -(k cc + c (cc - cc_prev) / dt) n
// with stiffness (k + c / dt) n n^T where cc > 1e-15, and the coating friction (return mapping on the
// coating surface with p_n = k cc, k_t = k * ratio; an uncompressed pair's history reset) with force
// -(q0 t1 + q1 t2) and stiffness T D T^T.  The coating state is read and updated in the pair table.
template <typename T, typename ST>
XK_D void coating_epilogue(const xk_contact_params& cp, const ST* __restrict__ prev_a,
                           ST* __restrict__ z_t, ST* __restrict__ qtn_a, ST* __restrict__ diss_a,
                           uint8_t* __restrict__ stick_a, long long i, long long cap, T cc, T s, T t, const T* n,
                           const T* t1, const T* t2, const T (*du)[3], T* v, T* B) {
  const T k = (T)cp.coat_k, c = (T)cp.coat_c, dt = (T)cp.coat_dt;
  const bool visc = cp.coat_c > 0.0 && cp.coat_dt > 0.0;
  const T prev = (T)prev_a[i];
  if (!(cc <= T(0) && prev <= T(0))) {  // forces (strategy.py:97-143)
    T f = k * cc;
    if (visc) f += c * ((cc - prev) / dt);
    if (!(my_abs<T>(f) < T(1e-30)))
      for (int q = 0; q < 3; ++q) v[q] -= f * n[q];
  }
  if (cc > T(1e-15)) {  // stiffness (strategy.py:145-196)
    const T k_eff = visc ? k + c / dt : k;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) B[3 * a + b] += k_eff * n[a] * n[b];
  }
  if (!(cp.coat_mu > 0.0)) return;
  const T k_t = k * (T)cp.coat_kt_ratio, mu = (T)cp.coat_mu;
  if (cc <= T(0)) {  // friction_forces (strategy.py:198-288): no coating contact, history reset
    z_t[i] = ST(0);
    z_t[cap + i] = ST(0);
    stick_a[i] = 1;
    qtn_a[i] = ST(0);
    diss_a[i] = ST(0);
    return;
  }
  const T p_n = k * cc;
  T rel[3];
  for (int q = 0; q < 3; ++q) rel[q] = ((T(1) - t) * du[2][q] + t * du[3][q]) - ((T(1) - s) * du[0][q] + s * du[1][q]);
  const T d0 = dot3(rel, t1), d1 = dot3(rel, t2);
  const T tr0 = (T)z_t[i] + k_t * d0, tr1 = (T)z_t[cap + i] + k_t * d1;
  const T qn = my_sqrt<T>(tr0 * tr0 + tr1 * tr1);
  const T fy = mu * p_n;
  const bool stick = qn <= fy;
  const T q0 = stick ? tr0 : fy * tr0 / qn, q1 = stick ? tr1 : fy * tr1 / qn;
  z_t[i] = (ST)q0;
  z_t[cap + i] = (ST)q1;
  stick_a[i] = stick ? 1 : 0;
  qtn_a[i] = (ST)qn;
  diss_a[i] = (ST)(q0 * d0 + q1 * d1);
  for (int q = 0; q < 3; ++q) v[q] -= q0 * t1[q] + q1 * t2[q];
  // friction_stiffness (strategy.py:290-370): D from _tangent_2x2_core on the updated state
  T D00 = k_t, D01 = T(0), D11 = k_t;
  const T zn = my_sqrt<T>(q0 * q0 + q1 * q1);
  if (!stick && zn >= T(1e-30) && qn >= T(1e-30)) {
    const T h0 = q0 / zn, h1 = q1 / zn, ratio = (mu * p_n) / qn;
    D00 = ratio * k_t * (T(1) - h0 * h0);
    D01 = ratio * k_t * (T(0) - h0 * h1);
    D11 = ratio * k_t * (T(1) - h1 * h1);
  }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      B[3 * a + b] += (t1[a] * D00 + t2[a] * D01) * t1[b] + (t1[a] * D01 + t2[a] * D11) * t2[b];
}

// Pairs that cannot contribute in this increment: only the frozen narrowphase,
// which the reference runs on every pair (_newton_steps.py:91-94) and which
// carries the frame transport history.
template <int P>
__global__ void __launch_bounds__(PAIR_T) k_pair_other(xk_mesh m, xk_pairs p, const int32_t* __restrict__ others,
                                                       int n_o, const double* __restrict__ u) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n_o) return;
  const int i = others[o];
  int nd[4];
  const int ea = p.ea[i], eb = p.eb[i];
  nd[0] = m.conn[2 * ea]; nd[1] = m.conn[2 * ea + 1]; nd[2] = m.conn[2 * eb]; nd[3] = m.conn[2 * eb + 1];
  double s, t, gap, n[3], t1[3], t2[3];
  pair_narrow<P>(m, p, i, nd, u, s, t, gap, n, t1, t2);
}

// Contributing pairs: narrowphase, Huber normal force, Coulomb return mapping
// and the pair tangent, one record (s, t, v, B) per member.
// COAT: the coated-wire epilogue is compiled in (a launch with coating selects it), so the plain
// kernel keeps its registers.
template <int P, int OUT, bool COAT>
__global__ void __launch_bounds__(PAIR_T) k_pair_member(xk_mesh m, xk_pairs p, const int32_t* __restrict__ members,
                                                        const int32_t* __restrict__ mnodes, int n_m,
                                                        const double* __restrict__ u, const double* __restrict__ u_ref,
                                                        xk_contact_params cp, int stages,
                                                        typename Prec<P>::T* __restrict__ rec, long long rs) {
  typedef typename Prec<P>::T T;
  const int mi = blockIdx.x * blockDim.x + threadIdx.x;
  if (mi >= n_m) return;
  const int i = members[mi];
  const long long cap = p.cap;
  int nd[4];
  for (int k = 0; k < 4; ++k) nd[k] = mnodes[4LL * mi + k];
  uint8_t status = p.status[i];
  double p_n = p.p_n[i];
  const double ra = m.radii[p.ea[i]], rb = m.radii[p.eb[i]];
  double s, t, gap, n[3], t1[3], t2[3];
  if (stages & XK_STAGE_NARROW) {
    pair_narrow<P>(m, p, i, nd, u, s, t, gap, n, t1, t2);
  } else {
    s = p.s[i];
    t = p.t[i];
    gap = p.gap[i];
    load3(p.normal, cap, i, n);
    load3(p.t1, cap, i, t1);
    load3(p.t2, cap, i, t2);
  }
  const double dh = cp.smoothing_delta > 0.0 ? cp.k_pen / cp.smoothing_delta : 0.0;
  const double xpen = cp.k_pen * (-gap);
  T vn[3] = {T(0), T(0), T(0)}, vf[3] = {T(0), T(0), T(0)};
  const T nT[3] = {(T)n[0], (T)n[1], (T)n[2]};
  const T t1T[3] = {(T)t1[0], (T)t1[1], (T)t1[2]};
  const T t2T[3] = {(T)t2[0], (T)t2[1], (T)t2[2]};
  // ---------------------------------------------------------------- normal force
  if ((stages & XK_STAGE_NORMAL) && status != ST_INACTIVE) {
    p_n = huber(xpen, dh);
    p.p_n[i] = p_n;
    if (p_n > 1e-30)
      for (int k = 0; k < 3; ++k) vn[k] = (T)p_n * nT[k];
  }
  // ---------------------------------------------------------------- friction
  double kt = p.k_t[i];
  double zt0 = p.z_t[i], zt1 = p.z_t[cap + i];
  double qtn = p.q_trial_norm[i];
  bool stick = p.stick[i] != 0;
  const double mu_eff = m.mu ? m.mu[p.ea[i]] : cp.mu_eff;
  const bool fproc = (p_n > 0.0) && (mu_eff > 0.0);
  if ((stages & XK_STAGE_FRICTION) && fproc) {
    if (p.k_pen[i] <= 0.0) {
      p.k_pen[i] = cp.k_pen;
      kt = cp.k_pen * cp.k_t_ratio;
      p.k_t[i] = kt;
    }
    T du[4][3];
    for (int k = 0; k < 4; ++k)
      for (int c = 0; c < 3; ++c) {
        const long long dof = 6LL * nd[k] + c;
        du[k][c] = (T)(u_ref ? u[dof] - u_ref[dof] : u[dof]);
      }
    const T sT = (T)s, tT = (T)t;
    T dr[3];
    for (int c = 0; c < 3; ++c)
      dr[c] = ((T(1) - tT) * du[2][c] + tT * du[3][c]) - ((T(1) - sT) * du[0][c] + sT * du[1][c]);
    const T d0 = dot3(dr, t1T), d1 = dot3(dr, t2T);
    const T ktT = (T)kt;
    const T q0 = (T)zt0 + ktT * d0, q1 = (T)zt1 + ktT * d1;
    const T qn = my_sqrt<T>(q0 * q0 + q1 * q1);
    const T fy = (T)mu_eff * (T)p_n;
    stick = qn <= fy;
    T r0 = q0, r1 = q1;
    if (!stick) { r0 = fy * q0 / qn; r1 = fy * q1 / qn; }
    zt0 = r0;
    zt1 = r1;
    qtn = qn;
    p.z_t[i] = zt0;
    p.z_t[cap + i] = zt1;
    p.stick[i] = stick ? 1 : 0;
    p.q_trial_norm[i] = qtn;
    p.dissipation[i] = (double)(r0 * d0 + r1 * d1);
    status = stick ? ST_ACTIVE : ST_SLIDING;
    p.status[i] = status;
    if (my_sqrt<T>(r0 * r0 + r1 * r1) >= T(1e-30)) {
      const T a0 = my_abs<T>(r0) < T(1e-30) ? T(0) : r0, a1 = my_abs<T>(r1) < T(1e-30) ? T(0) : r1;
      for (int k = 0; k < 3; ++k) vf[k] = a0 * t1T[k] + a1 * t2T[k];
    }
  }
  // ---------------------------------------------------------------- tangent
  T Bn[9], Bf[9];
  for (int k = 0; k < 9; ++k) { Bn[k] = T(0); Bf[k] = T(0); }
  if ((stages & XK_STAGE_TANGENT) && status != ST_INACTIVE) {
    const double dist = (gap + ra) + rb;
    const double hd = huber_deriv(xpen, dh);
    if (!(hd < 1e-30 && p_n < 1e-30)) {
      const T wm = (T)(hd * cp.k_pen);
      const T wg = (T)(dist > 1e-15 ? p_n / dist : 0.0);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          const T nn = nT[a] * nT[b];
          Bn[3 * a + b] = wm * nn - wg * ((a == b ? T(1) : T(0)) - nn);
        }
    }
    const T q0 = (T)zt0, q1 = (T)zt1;
    const T qnorm = my_sqrt<T>(q0 * q0 + q1 * q1);
    if (fproc && qnorm >= T(1e-30)) {
      const T ktT = (T)kt;
      T D00 = ktT, D01 = T(0), D11 = ktT;
      if (!stick && (T)qtn >= T(1e-30)) {
        const T qh0 = q0 / qnorm, qh1 = q1 / qnorm;
        const T ratio = (T)mu_eff * (T)p_n / (T)qtn;
        D00 = ratio * ktT * (T(1) - qh0 * qh0);
        D01 = -ratio * ktT * qh0 * qh1;
        D11 = ratio * ktT * (T(1) - qh1 * qh1);
      }
      if (my_abs<T>(D00) < T(1e-30)) D00 = T(0);
      if (my_abs<T>(D01) < T(1e-30)) D01 = T(0);
      if (my_abs<T>(D11) < T(1e-30)) D11 = T(0);
      const bool geo = (dist >= 1e-15) && !(my_abs<T>(q0) < T(1e-30) && my_abs<T>(q1) < T(1e-30));
      const T idist = geo ? (T)(1.0 / dist) : T(0);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          const T mat = D00 * t1T[a] * t1T[b] + D01 * (t1T[a] * t2T[b] + t2T[a] * t1T[b]) + D11 * t2T[a] * t2T[b];
          const T M = -q0 * nT[a] * t1T[b] - q1 * t2T[a] * nT[b];
          Bf[3 * a + b] = mat + idist * M;
        }
      // + q2 [t1]x^T
      Bf[1] += idist * q1 * t1T[2];
      Bf[2] -= idist * q1 * t1T[1];
      Bf[3] -= idist * q1 * t1T[2];
      Bf[5] += idist * q1 * t1T[0];
      Bf[6] += idist * q1 * t1T[1];
      Bf[7] -= idist * q1 * t1T[0];
    }
  }
  // ---------------------------------------------------------------- coating (coated wires)
  T vc[3] = {T(0), T(0), T(0)}, Bc[9];
  for (int k = 0; k < 9; ++k) Bc[k] = T(0);
  constexpr int ALL = XK_STAGE_NORMAL | XK_STAGE_FRICTION | XK_STAGE_TANGENT;
  if (COAT && OUT == XK_OUT_COMBINED && m.core_radii && p.coat_cc && (stages & ALL) == ALL) {
    T duc[4][3];
    for (int k = 0; k < 4; ++k)
      for (int c = 0; c < 3; ++c) {
        const long long dof = 6LL * nd[k] + c;
        duc[k][c] = (T)(u_ref ? u[dof] - u_ref[dof] : u[dof]);
      }
    coating_epilogue<T, double>(cp, p.coat_cc_prev, p.coat_z_t, p.coat_qtn, p.coat_diss, p.coat_stick, i, cap,
                                (T)p.coat_cc[i], (T)s, (T)t, nT, t1T, t2T, duc, vc, Bc);
  }
  // ---------------------------------------------------------------- record
  T* r = rec + (long long)mi * rs;  // array-of-structs record, rs values per member
  if (OUT == XK_OUT_COMBINED) {
    for (int k = 0; k < 9; ++k) r[XK_REC_B + k] = (Bn[k] - Bf[k]) + Bc[k];
    r[XK_REC_S] = (T)s;
    r[XK_REC_S + 1] = (T)t;
    for (int k = 0; k < 3; ++k) r[XK_REC_V + k] = (vn[k] + vf[k]) + vc[k];
    r[14] = T(0);
    r[15] = T(0);
  } else {
    r[0] = (T)s;
    r[1] = (T)t;
    if (stages & XK_STAGE_NORMAL)
      for (int k = 0; k < 3; ++k) r[2 + k] = vn[k];
    if (stages & XK_STAGE_FRICTION)
      for (int k = 0; k < 3; ++k) r[5 + k] = vf[k];
    if (stages & XK_STAGE_TANGENT) {
      for (int k = 0; k < 9; ++k) r[8 + k] = Bn[k];
      for (int k = 0; k < 9; ++k) r[17 + k] = Bf[k];
    }
  }
}

// ===========================================================================
// Mixed fast path: no double-precision instruction per pair.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the per-iteration
// pair kernels of the mixed path use float only.  The one quantity float
// cannot resolve is the gap dist - (r_a + r_b): dist is about r_a + r_b and
// the gap is a few tenths of a percent of it.  It is taken in float-float
// ("df") arithmetic: error-free two-sum / two-product transformations on the
// FP32 pipe, from node positions that xk_nodes_prepare splits once per
// iteration into a float high part and a float remainder.
// ===========================================================================

struct df {
  float h, l;
};
XK_D df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
XK_D df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
XK_D df df_sub(df a, df b) {
  const df s = two_sum(a.h, -b.h);
  return fast_two_sum(s.h, s.l + (a.l - b.l));
}
XK_D df df_add(df a, df b) {
  const df s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, s.l + (a.l + b.l));
}
XK_D df df_mulf(df a, float b) {
  const float p = a.h * b;
  const float e = fmaf(a.h, b, -p);
  return fast_two_sum(p, fmaf(a.l, b, e));
}

// One thread per node.  The double arithmetic here (X + u, its split, the conversions) runs
// on the FP64 pipe, a small fraction of the FP32 rate on this GPU, so each value is converted
// once.  VEC: u and u_ref are 16-byte aligned and read as double2 (48 bytes per node).
template <bool VEC>
__global__ void k_nodes_prepare(xk_mesh m, const double* __restrict__ u, const double* __restrict__ u_ref,
                                float* __restrict__ n32) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.n_nodes) return;
  double uv[6], ur[3] = {0.0, 0.0, 0.0};
  if (VEC) {
    const double2* up = reinterpret_cast<const double2*>(u + 6LL * v);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double2 a = __ldg(up + i);
      uv[2 * i] = a.x;
      uv[2 * i + 1] = a.y;
    }
    if (u_ref) {
      const double2* rp = reinterpret_cast<const double2*>(u_ref + 6LL * v);
      const double2 a = __ldg(rp), b = __ldg(rp + 1);
      ur[0] = a.x; ur[1] = a.y; ur[2] = b.x;
    }
  } else {
#pragma unroll
    for (int c = 0; c < 6; ++c) uv[c] = u[6LL * v + c];
    if (u_ref)
      for (int c = 0; c < 3; ++c) ur[c] = u_ref[6LL * v + c];
  }
  float N[16];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double x = m.X[3LL * v + c] + uv[c];
    const float h = xk_d2f(x);
    N[c] = h;
    N[3 + c] = xk_d2f(x - xk_f2d(h));
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) N[6 + c] = xk_d2f(uv[c]);
#pragma unroll
  for (int c = 0; c < 3; ++c) N[12 + c] = xk_d2f(u_ref ? uv[c] - ur[c] : uv[c]);
  N[15] = 0.0f;
  float4* out = reinterpret_cast<float4*>(n32 + (long long)v * XK_NODE32_STRIDE);
#pragma unroll
  for (int i = 0; i < 4; ++i) out[i] = make_float4(N[4 * i], N[4 * i + 1], N[4 * i + 2], N[4 * i + 3]);
}

__global__ void k_pairs_to32(xk_mesh m, xk_pairs p, xk_contact_pattern pat, xk_pairs32 q) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= q.n) return;
  const bool mem = j < pat.n_members;
  const int i = mem ? pat.members[j] : pat.others[j - pat.n_members];
  const long long cp = p.cap, cq = q.cap;
  q.pair[j] = i;
  if (q.slot) q.slot[i] = j;
  const int ea = p.ea[i], eb = p.eb[i];
  q.nodes[4LL * j] = m.conn[2 * ea];
  q.nodes[4LL * j + 1] = m.conn[2 * ea + 1];
  q.nodes[4LL * j + 2] = m.conn[2 * eb];
  q.nodes[4LL * j + 3] = m.conn[2 * eb + 1];
  const bool coat = q.coat_total && m.core_radii && p.coat_cc;  // coated wires: the gap between the cores
  const double R = coat ? m.core_radii[ea] + m.core_radii[eb] : m.radii[ea] + m.radii[eb];
  const float rh = xk_d2f(R);
  q.rad[2LL * j] = rh;
  q.rad[2LL * j + 1] = xk_d2f(R - xk_f2d(rh));
  if (coat) {
    q.coat_total[j] = xk_d2f(coat_total_of(m, ea, eb));
    q.coat_cc[j] = xk_d2f(p.coat_cc[i]);
    q.coat_cc_prev[j] = xk_d2f(p.coat_cc_prev[i]);
    q.coat_z_t[j] = xk_d2f(p.coat_z_t[i]);
    q.coat_z_t[cq + j] = xk_d2f(p.coat_z_t[cp + i]);
    q.coat_qtn[j] = xk_d2f(p.coat_qtn[i]);
    q.coat_diss[j] = xk_d2f(p.coat_diss[i]);
    q.coat_stick[j] = p.coat_stick[i];
  }
  q.s[j] = xk_d2f(p.s[i]); q.t[j] = xk_d2f(p.t[i]); q.gap[j] = xk_d2f(p.gap[i]);
  for (int c = 0; c < 3; ++c) {
    q.normal[c * cq + j] = xk_d2f(p.normal[c * cp + i]);
    q.t1[c * cq + j] = xk_d2f(p.t1[c * cp + i]);
    q.t2[c * cq + j] = xk_d2f(p.t2[c * cp + i]);
  }
  q.p_n[j] = xk_d2f(p.p_n[i]);
  q.z_t[j] = xk_d2f(p.z_t[i]); q.z_t[cq + j] = xk_d2f(p.z_t[cp + i]);
  q.q_trial_norm[j] = xk_d2f(p.q_trial_norm[i]); q.dissipation[j] = xk_d2f(p.dissipation[i]);
  q.k_pen[j] = xk_d2f(p.k_pen[i]); q.k_t[j] = xk_d2f(p.k_t[i]);
  q.status[j] = p.status[i]; q.stick[j] = p.stick[i];
  if (q.mu && m.mu) q.mu[j] = xk_d2f(m.mu[ea]);
}

// BY_PAIR: a thread per pair i of the FP64 table (j from q.slot; the writes coalesce, and the reads come
// from two ascending runs of slots, members' and others'); else a thread per slot j
template <bool BY_PAIR>
__global__ void k_pairs_from32(xk_pairs32 q, xk_pairs p) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= q.n) return;
  const int j = BY_PAIR ? q.slot[t] : t;
  const int i = BY_PAIR ? t : q.pair[j];
  const long long cp = p.cap, cq = q.cap;
  p.s[i] = xk_f2d(q.s[j]); p.t[i] = xk_f2d(q.t[j]); p.gap[i] = xk_f2d(q.gap[j]);
  float n[3], t1[3], t2[3];
  for (int c = 0; c < 3; ++c) {
    n[c] = q.normal[c * cq + j];
    t1[c] = q.t1[c * cq + j];
    t2[c] = q.t2[c * cq + j];
  }
  if (j >= q.n_members) cross3(n, t1, t2);  // the other-pair kernel does not store t2
  for (int c = 0; c < 3; ++c) {
    p.normal[c * cp + i] = xk_f2d(n[c]);
    p.t1[c * cp + i] = xk_f2d(t1[c]);
    p.t2[c * cp + i] = xk_f2d(t2[c]);
  }
  p.p_n[i] = xk_f2d(q.p_n[j]);
  p.z_t[i] = xk_f2d(q.z_t[j]); p.z_t[cp + i] = xk_f2d(q.z_t[cq + j]);
  p.q_trial_norm[i] = xk_f2d(q.q_trial_norm[j]); p.dissipation[i] = xk_f2d(q.dissipation[j]);
  p.k_pen[i] = xk_f2d(q.k_pen[j]); p.k_t[i] = xk_f2d(q.k_t[j]);
  p.status[i] = q.status[j]; p.stick[i] = q.stick[j];
  if (q.coat_total && p.coat_cc) {
    p.coat_cc[i] = xk_f2d(q.coat_cc[j]);
    p.coat_cc_prev[i] = xk_f2d(q.coat_cc_prev[j]);
    p.coat_z_t[i] = xk_f2d(q.coat_z_t[j]);
    p.coat_z_t[cp + i] = xk_f2d(q.coat_z_t[cq + j]);
    p.coat_qtn[i] = xk_f2d(q.coat_qtn[j]);
    p.coat_diss[i] = xk_f2d(q.coat_diss[j]);
    p.coat_stick[i] = q.coat_stick[j];
  }
}

XK_D float clamp01f(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

// Closest point and gap of one pair from prepared nodes; frame transported from
// the previous float frame.  Near-parallel pairs fall back to the exact routine.
// With DF the difference vector and the gap are taken in float-float arithmetic
// (contributing pairs: the gap drives the normal force).  Without it they are
// plain float from the exact float differences of the split positions, an
// absolute gap error of a few float roundings of the segment length (1e-7 mm
// at 0.5 mm wires): enough for pairs that carry no force in the increment,
// whose gap the next detection recomputes exactly.
// With DEFER the near-parallel case is not handled: the function returns true at once and leaves
// every output untouched (the caller hands the pair to a kernel compiled without DEFER).
template <bool DF, bool DEFER = false>
XK_D bool narrow32(const float* __restrict__ n32, const int* nd, df R, float& s, float& t, float& gap, float* n,
                   float* pt1_io, float* t2) {
  df x[4][3];
  for (int k = 0; k < 4; ++k) {
    float N[8];  // x_hi (3), x_lo (3) and two values not used here: one 256-bit load of a 64-byte record
    ldg8(n32 + (long long)nd[k] * XK_NODE32_STRIDE, N);
    x[k][0] = {N[0], N[3]};
    x[k][1] = {N[1], N[4]};
    x[k][2] = {N[2], N[5]};
  }
  float fa[3], fb[3], fw[3];
  for (int c = 0; c < 3; ++c) {
    fa[c] = (x[1][c].h - x[0][c].h) + (x[1][c].l - x[0][c].l);
    fb[c] = (x[3][c].h - x[2][c].h) + (x[3][c].l - x[2][c].l);
    fw[c] = (x[0][c].h - x[2][c].h) + (x[0][c].l - x[2][c].l);
  }
  const float a = dot3(fa, fa), b = dot3(fa, fb), c = dot3(fb, fb), d = dot3(fa, fw), e = dot3(fb, fw);
  const float ac = a * c, det = ac - b * b;
  float nrm[3];
  if (DEFER && !(det > 1e-3f * ac)) return true;
  if (!(det > 1e-3f * ac)) {
    // rare: near-parallel or degenerate segments, exact double routine on the node records read
    // again (so that the split positions need not stay live through the common path)
    double xd[4][3], sd, td, dist, nd3[3], diff[3];
    for (int k = 0; k < 4; ++k) {
      float N[8];
      ldg8(n32 + (long long)nd[k] * XK_NODE32_STRIDE, N);
      for (int q = 0; q < 3; ++q) xd[k][q] = (double)N[q] + (double)N[3 + q];
    }
    closest_exact(xd[0], xd[1], xd[2], xd[3], sd, td, dist, nd3, diff);
    s = (float)sd;
    t = (float)td;
    gap = (float)(dist - ((double)R.h + (double)R.l));
    for (int q = 0; q < 3; ++q) nrm[q] = (float)nd3[q];
  } else {
    const float idet = 1.0f / det;
    const float su = (b * e - c * d) * idet, tu = (a * e - b * d) * idet;
    float sf = clamp01f(su), tf = clamp01f(tu);
    if (su < 0.0f || su > 1.0f) tf = clamp01f((b * sf + e) / c);
    if (tu < 0.0f || tu > 1.0f) {
      sf = clamp01f((b * tf - d) / a);
      tf = clamp01f((b * sf + e) / c);
    }
    s = sf;
    t = tf;
    if (!DF) {
      float D[3];
      for (int q = 0; q < 3; ++q) D[q] = fmaf(-tf, fb[q], fmaf(sf, fa[q], fw[q]));
      const float dist = sqrtf(dot3(D, D));
      gap = (dist - R.h) - R.l;
      const float id = 1.0f / dist;
      for (int q = 0; q < 3; ++q) nrm[q] = D[q] * id;
      if (!(dist > 1e-30f)) { nrm[0] = 0.0f; nrm[1] = 0.0f; nrm[2] = 1.0f; }
    } else {
    // diff = (xA0 - xB0) + s (xA1 - xA0) - t (xB1 - xB0) in float-float
    df D[3];
    for (int q = 0; q < 3; ++q) {
      const df w0 = df_sub(x[0][q], x[2][q]);
      const df dA = df_sub(x[1][q], x[0][q]);
      const df dB = df_sub(x[3][q], x[2][q]);
      D[q] = df_sub(df_add(w0, df_mulf(dA, sf)), df_mulf(dB, tf));
    }
    // |D|^2 with the squares of the high parts taken exactly
    df S = {0.0f, 0.0f};
    float cross_terms = 0.0f;
    for (int q = 0; q < 3; ++q) {
      const float p = D[q].h * D[q].h;
      const df sq = {p, fmaf(D[q].h, D[q].h, -p)};
      S = df_add(S, sq);
      cross_terms = fmaf(2.0f * D[q].h, D[q].l, cross_terms);
    }
    S = fast_two_sum(S.h, S.l + cross_terms);
    const float dh = sqrtf(S.h);
    const float dl = (fmaf(-dh, dh, S.h) + S.l) / (2.0f * dh);
    gap = (dh - R.h) + (dl - R.l);
    const float id = 1.0f / dh;
    for (int q = 0; q < 3; ++q) nrm[q] = D[q].h * id;
    if (!(dh > 1e-30f)) { nrm[0] = 0.0f; nrm[1] = 0.0f; nrm[2] = 1.0f; }
    }
  }
  // frame transport (float)
  float pn[3] = {n[0], n[1], n[2]};  // previous normal on entry
  float pt1[3] = {pt1_io[0], pt1_io[1], pt1_io[2]};
  const float inv = rsqrtf(fmaxf(dot3(nrm, nrm), 1e-30f));
  for (int q = 0; q < 3; ++q) n[q] = nrm[q] * inv;
  const bool has_t1 = dot3(pt1, pt1) > 1e-20f, has_n = dot3(pn, pn) > 1e-20f;
  bool done = false;
  float t1[3];
  if (has_t1) {
    float tr[3] = {pt1[0], pt1[1], pt1[2]};
    if (has_n) {
      const float ip = rsqrtf(dot3(pn, pn));
      const float no[3] = {pn[0] * ip, pn[1] * ip, pn[2] * ip};
      float v[3], vx[3], vvx[3];
      cross3(no, n, v);
      const float cv = dot3(no, n), s2 = dot3(v, v);
      if (cv > 0.0f || s2 >= 1e-24f) {
        cross3(v, pt1, vx);
        cross3(v, vx, vvx);
        const float f = cv > 0.0f ? 1.0f / (1.0f + cv) : (1.0f - cv) / s2;
        for (int q = 0; q < 3; ++q) tr[q] = pt1[q] + vx[q] + f * vvx[q];
      }
    }
    const float dn = dot3(tr, n);
    const float raw[3] = {tr[0] - dn * n[0], tr[1] - dn * n[1], tr[2] - dn * n[2]};
    const float r2 = dot3(raw, raw);
    if (r2 > 1e-20f) {
      const float ir = rsqrtf(r2);
      for (int q = 0; q < 3; ++q) t1[q] = raw[q] * ir;
      done = true;
    }
  }
  if (!done) {
    float ref[3] = {0.f, 0.f, 0.f};
    const float a0 = fabsf(n[0]), a1 = fabsf(n[1]), a2 = fabsf(n[2]);
    ref[(a0 <= a1 && a0 <= a2) ? 0 : (a1 <= a2 ? 1 : 2)] = 1.0f;
    const float dn = dot3(ref, n);
    const float raw[3] = {ref[0] - dn * n[0], ref[1] - dn * n[1], ref[2] - dn * n[2]};
    const float ir = rsqrtf(fmaxf(dot3(raw, raw), 1e-30f));
    for (int q = 0; q < 3; ++q) t1[q] = raw[q] * ir;
  }
  cross3(n, t1, t2);
  for (int q = 0; q < 3; ++q) pt1_io[q] = t1[q];
  return false;
}

XK_D void load3f(const float* base, long long stride, long long i, float* v) {
  v[0] = base[i];
  v[1] = base[stride + i];
  v[2] = base[2 * stride + i];
}
XK_D void store3f(float* base, long long stride, long long i, const float* v) {
  base[i] = v[0];
  base[stride + i] = v[1];
  base[2 * stride + i] = v[2];
}

// Detection narrowphase of the mixed engine.  Every pair's closest point, gap and frame are
// taken in float from the split node positions (narrow32 without float-float), and the
// active-set update (_manager_process.py:475-494) is decided on that gap wherever it cannot
// differ from the exact one: the pair goes to the exact FP64 routine instead (appended to
// `list`) when it is near-parallel, on coated wires, or when its float gap lies within eps of
// [g_on, g_off].  eps bounds |gap_f - gap|: the inputs are the differences of the split positions
// rounded once (relative 2^-24 of the scale, the largest |component| of the two segments and of
// their offset), the 2x2 solve runs only with det > 1e-3 ac, so the parameter error is below
// about 8e3 2^-24 and the distance at the computed parameters exceeds the segment distance by at
// most the square of the resulting point error over twice the distance; the rounding of the
// difference vector and its norm adds a few units of 2^-24 scale.  eps = 2e-5 scale + that square
// term over (r_a + r_b) covers both with a wide margin.  The frames of the pairs decided in float
// are transported in float (the per-iteration narrowphase of the mixed path does the same).
// g_on_lo / g_off_hi: the thresholds rounded outward to float.  The band test, the error bound and
// the decisions are all in float (FP64 runs at 1/64 of the FP32 rate on this GPU); the bound is
// rounded up and the band's ends rounded outward, so that a gap outside the band lies on the same side
// of the thresholds as the exact one.
__global__ void __launch_bounds__(PAIR_T) k_narrow_screen(xk_mesh m, xk_pairs p, const float* __restrict__ n32,
                                                         float g_on_lo, float g_off_hi, int allow_deact,
                                                         int32_t* __restrict__ list) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const long long cap = p.cap;
  const int ea = p.ea[i], eb = p.eb[i];
  const PairNodes pn = pair_nodes(m, ea, eb);
  const int nd[4] = {pn.n[0], pn.n[1], pn.n[2], pn.n[3]};
  const double rs = xadd(m.radii[ea], m.radii[eb]);
  const float rh = xk_d2f(rs);
  const df R = {rh, xk_d2f(rs - xk_f2d(rh))};
  float scale = 0.0f;
  {
    float xh[4][3];
    for (int k = 0; k < 4; ++k) {
      float N[8];
      ldg8(n32 + (long long)nd[k] * XK_NODE32_STRIDE, N);
      for (int c = 0; c < 3; ++c) xh[k][c] = N[c];
    }
    for (int c = 0; c < 3; ++c)
      scale = fmaxf(scale, fmaxf(fabsf(xh[1][c] - xh[0][c]), fmaxf(fabsf(xh[3][c] - xh[2][c]),
                                                                   fabsf(xh[0][c] - xh[2][c]))));
  }
  float n[3], t1[3], t2[3], sf, tf, gf;
  {
    double v[3];
    load3(p.normal, cap, i, v);
    for (int c = 0; c < 3; ++c) n[c] = xk_d2f(v[c]);
    load3(p.t1, cap, i, v);
    for (int c = 0; c < 3; ++c) t1[c] = xk_d2f(v[c]);
  }
  const bool deferred = m.core_radii != nullptr || narrow32<false, true>(n32, nd, R, sf, tf, gf, n, t1, t2);
  const float u24 = 5.9604645e-8f;  // 2^-24
  const float pe = 8.0e3f * u24 * scale;
  // eps = 2e-5 scale + pe^2 / (2 r_s), raised by 2^-20 of itself for its own roundings (the fast
  // division's 2 ulp and the float constants included)
  const float eps = (2e-5f * scale + __fdividef(pe * pe, 2.0f * rh)) * (1.0f + 9.5367432e-7f);
  const float lo = __fsub_rd(g_on_lo, eps), hi = __fadd_ru(g_off_hi, eps);
  if (deferred || (gf >= lo && gf <= hi)) {
    list[1 + atomicAdd(list, 1)] = i;
    return;
  }
  p.s[i] = xk_f2d(sf);
  p.t[i] = xk_f2d(tf);
  p.gap[i] = xk_f2d(gf);
  const double nn[3] = {xk_f2d(n[0]), xk_f2d(n[1]), xk_f2d(n[2])};
  const double tt1[3] = {xk_f2d(t1[0]), xk_f2d(t1[1]), xk_f2d(t1[2])};
  const double tt2[3] = {xk_f2d(t2[0]), xk_f2d(t2[1]), xk_f2d(t2[2])};
  store3(p.normal, cap, i, nn);
  store3(p.t1, cap, i, tt1);
  store3(p.t2, cap, i, tt2);
  const uint8_t st = p.status[i];  // gf is outside [lo, hi]: the exact gap is on the same side of both thresholds
  if (st == ST_INACTIVE) {
    if (gf < lo) p.status[i] = ST_ACTIVE;
  } else if (allow_deact && gf > hi) {
    p.status[i] = ST_INACTIVE;
  }
}

// The exact detection narrowphase of the pairs the screen listed (list[0] of them), grid-stride.
__global__ void k_narrow_exact_list(xk_mesh m, xk_pairs p, const double* __restrict__ u, double g_on, double g_off,
                                    int allow_deact, const int32_t* __restrict__ list) {
  const int n = list[0];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    narrow_exact_one(m, p, u, g_on, g_off, allow_deact, 1, list[1 + k]);
}

// A deferral list: [count, done, slots...].  The pair kernel appends to it; its deferred kernel
// reads the count, works through the slots grid-stride, and its last CTA to finish (found with
// the `done` counter after every CTA has read the count) sets both words back to zero for the
// next launch, so the list needs no reset of its own.
constexpr int DEFER_SLOTS = 2;

// Other-pair narrowphase of slot j.  DEFER: near-parallel pairs are appended to q.defer instead
// (any order: each is then computed on its own by k_pair_other32_deferred).
template <bool DEFER>
XK_D void other32(const xk_pairs32& q, const float* __restrict__ n32, int j) {
  const long long cq = q.cap;
  const int4 nd4 = __ldg(reinterpret_cast<const int4*>(q.nodes) + j);
  const int nd[4] = {nd4.x, nd4.y, nd4.z, nd4.w};
  const float2 R2 = __ldg(reinterpret_cast<const float2*>(q.rad) + j);
  float s, t, gap, n[3], t1[3], t2[3];
  load3f(q.normal, cq, j, n);
  load3f(q.t1, cq, j, t1);
  if (narrow32<false, DEFER>(n32, nd, {R2.x, R2.y}, s, t, gap, n, t1, t2)) {
    q.defer[DEFER_SLOTS + atomicAdd(q.defer, 1)] = j;
    return;
  }
  q.s[j] = s;
  q.t[j] = t;
  q.gap[j] = gap;
  store3f(q.normal, cq, j, n);
  store3f(q.t1, cq, j, t1);
  // t2 = n x t1 is not stored for these pairs; k_pairs_from32 forms it
}

template <bool DEFER>
__global__ void __launch_bounds__(PAIR_T) k_pair_other32(xk_pairs32 q, const float* __restrict__ n32) {
  const int j = q.n_members + blockIdx.x * blockDim.x + threadIdx.x;
  if (j < q.n) other32<DEFER>(q, n32, j);
}

XK_D bool last_cta_done(int32_t* done) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(done, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  return last;
}

// The deferred (near-parallel) other pairs, grid-stride over the list.
__global__ void __launch_bounds__(PAIR_T) k_pair_other32_deferred(xk_pairs32 q, const float* __restrict__ n32) {
  int32_t* list = q.defer;
  const int cnt = *(volatile int32_t*)list;
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < cnt; x += gridDim.x * blockDim.x)
    other32<false>(q, n32, list[DEFER_SLOTS + x]);
  if (last_cta_done(list + 1) && threadIdx.x == 0) {
    list[0] = 0;
    list[1] = 0;
  }
}

// Member slot i (record i).  DEFER: a near-parallel member is appended to the member part of
// q.defer (after the cap + 2 words of the other pairs' list) and left to k_pair_member32_deferred.
template <bool DEFER>
XK_D void member32(const xk_pairs32& q, const float* __restrict__ n32, const xk_contact_params& cp,
                   float* __restrict__ rec, int i) {
  const int mi = i;
  const long long cq = q.cap;
  const int4 nd4 = __ldg(reinterpret_cast<const int4*>(q.nodes) + i);
  const int nd[4] = {nd4.x, nd4.y, nd4.z, nd4.w};
  const float2 R2 = __ldg(reinterpret_cast<const float2*>(q.rad) + i);
  const df R = {R2.x, R2.y};
  float s, t, gap, n[3], t1[3], t2[3];
  load3f(q.normal, cq, i, n);
  load3f(q.t1, cq, i, t1);
  if (narrow32<true, DEFER>(n32, nd, R, s, t, gap, n, t1, t2)) {
    int32_t* list = q.defer + (cq + DEFER_SLOTS);
    list[DEFER_SLOTS + atomicAdd(list, 1)] = i;
    return;
  }
  uint8_t status = q.status[i];
  q.s[i] = s;
  q.t[i] = t;
  q.gap[i] = gap;
  store3f(q.normal, cq, i, n);
  store3f(q.t1, cq, i, t1);
  store3f(q.t2, cq, i, t2);
  // normal force (Huber)
  // the parameters converted in integer arithmetic (a conversion instruction issues at the FP64 rate, and
  // every member thread needs them); smoothing_delta > 0 tested on its bits (positive, at most +inf)
  const float kpen = xk_d2f(cp.k_pen);
  const long long sd_bits = __double_as_longlong(cp.smoothing_delta);
  const float dh = (sd_bits > 0 && sd_bits <= 0x7ff0000000000000LL) ? xk_d2f(cp.k_pen / cp.smoothing_delta) : 0.0f;
  const float xpen = kpen * (-gap);
  float p_n = q.p_n[i];
  float vn[3] = {0.f, 0.f, 0.f}, vf[3] = {0.f, 0.f, 0.f};
  if (status != ST_INACTIVE) {
    p_n = (dh <= 0.0f) ? fmaxf(xpen, 0.0f)
                       : (xpen < -dh ? 0.0f : (xpen > dh ? xpen : (xpen + dh) * (xpen + dh) / (4.0f * dh)));
    q.p_n[i] = p_n;
    if (p_n > 1e-30f)
      for (int k = 0; k < 3; ++k) vn[k] = p_n * n[k];
  }
  // friction (Coulomb return mapping)
  const float mu = q.mu ? q.mu[i] : xk_d2f(cp.mu_eff);
  float kt = q.k_t[i];
  float zt0 = q.z_t[i], zt1 = q.z_t[cq + i];
  float qtn = q.q_trial_norm[i];
  bool stick = q.stick[i] != 0;
  const bool fproc = (p_n > 0.0f) && (mu > 0.0f);
  if (fproc) {
    if (q.k_pen[i] <= 0.0f) {
      q.k_pen[i] = kpen;
      kt = (float)(cp.k_pen * cp.k_t_ratio);
      q.k_t[i] = kt;
    }
    float du[4][3];
    for (int k = 0; k < 4; ++k) {
      const float4 d4 = __ldg(reinterpret_cast<const float4*>(n32 + (long long)nd[k] * XK_NODE32_STRIDE + 12));
      du[k][0] = d4.x; du[k][1] = d4.y; du[k][2] = d4.z;
    }
    float dr[3];
    for (int c = 0; c < 3; ++c) dr[c] = ((1.f - t) * du[2][c] + t * du[3][c]) - ((1.f - s) * du[0][c] + s * du[1][c]);
    const float d0 = dot3(dr, t1), d1 = dot3(dr, t2);
    const float q0 = zt0 + kt * d0, q1 = zt1 + kt * d1;
    const float qn = sqrtf(q0 * q0 + q1 * q1);
    const float fy = mu * p_n;
    stick = qn <= fy;
    float r0 = q0, r1 = q1;
    if (!stick) { r0 = fy * q0 / qn; r1 = fy * q1 / qn; }
    zt0 = r0; zt1 = r1; qtn = qn;
    q.z_t[i] = zt0;
    q.z_t[cq + i] = zt1;
    q.stick[i] = stick ? 1 : 0;
    q.q_trial_norm[i] = qtn;
    q.dissipation[i] = r0 * d0 + r1 * d1;
    status = stick ? ST_ACTIVE : ST_SLIDING;
    q.status[i] = status;
    if (sqrtf(r0 * r0 + r1 * r1) >= 1e-30f) {
      const float a0 = fabsf(r0) < 1e-30f ? 0.f : r0, a1 = fabsf(r1) < 1e-30f ? 0.f : r1;
      for (int k = 0; k < 3; ++k) vf[k] = a0 * t1[k] + a1 * t2[k];
    }
  }
  // pair tangent B = B_n - B_f
  float B[9];
  for (int k = 0; k < 9; ++k) B[k] = 0.f;
  // coated wires: the gap is between the cores; the geometric terms take gap + r_a + r_b as the
  // reference does (contact_force/strategy.py:230-236, friction/_assembly.py:203-204)
  const float ct = q.coat_total ? q.coat_total[i] : 0.0f;
  if (status != ST_INACTIVE) {
    const float dist = gap + ((R.h + R.l) + ct);
    const float hd = (dh <= 0.0f) ? (xpen > 0.0f ? 1.0f : 0.0f)
                                  : (xpen < -dh ? 0.0f : (xpen > dh ? 1.0f : (xpen + dh) / (2.0f * dh)));
    if (!(hd < 1e-30f && p_n < 1e-30f)) {
      const float wm = hd * kpen, wg = dist > 1e-15f ? p_n / dist : 0.0f;
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          const float nn = n[a] * n[b];
          B[3 * a + b] = wm * nn - wg * ((a == b ? 1.f : 0.f) - nn);
        }
    }
    const float qnorm = sqrtf(zt0 * zt0 + zt1 * zt1);
    if (fproc && qnorm >= 1e-30f) {
      float D00 = kt, D01 = 0.f, D11 = kt;
      if (!stick && qtn >= 1e-30f) {
        const float qh0 = zt0 / qnorm, qh1 = zt1 / qnorm, ratio = mu * p_n / qtn;
        D00 = ratio * kt * (1.f - qh0 * qh0);
        D01 = -ratio * kt * qh0 * qh1;
        D11 = ratio * kt * (1.f - qh1 * qh1);
      }
      const bool geo = (dist >= 1e-15f) && !(fabsf(zt0) < 1e-30f && fabsf(zt1) < 1e-30f);
      const float idist = geo ? 1.0f / dist : 0.0f;
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          const float mat = D00 * t1[a] * t1[b] + D01 * (t1[a] * t2[b] + t2[a] * t1[b]) + D11 * t2[a] * t2[b];
          const float M = -zt0 * n[a] * t1[b] - zt1 * t2[a] * n[b];
          B[3 * a + b] -= mat + idist * M;
        }
      const float g = idist * zt1;
      B[1] -= g * t1[2];
      B[2] += g * t1[1];
      B[3] += g * t1[2];
      B[5] -= g * t1[0];
      B[6] -= g * t1[1];
      B[7] += g * t1[0];
    }
  }
  if (q.coat_total) {  // Kelvin-Voigt coating, added to the record
    const float cc = fmaxf(0.0f, ct - gap);
    q.coat_cc[i] = cc;
    float duc[4][3];
    for (int k = 0; k < 4; ++k) {
      const float4 d4 = __ldg(reinterpret_cast<const float4*>(n32 + (long long)nd[k] * XK_NODE32_STRIDE + 12));
      duc[k][0] = d4.x; duc[k][1] = d4.y; duc[k][2] = d4.z;
    }
    float vc[3] = {0.f, 0.f, 0.f};
    coating_epilogue<float, float>(cp, q.coat_cc_prev, q.coat_z_t, q.coat_qtn, q.coat_diss, q.coat_stick, i, cq, cc,
                                   s, t, n, t1, t2, duc, vc, B);
    for (int k = 0; k < 3; ++k) vf[k] += vc[k];
  }
  float4* r = reinterpret_cast<float4*>(rec + (long long)mi * XK_REC_STRIDE_COMBINED);
  r[0] = make_float4(B[0], B[1], B[2], B[3]);
  r[1] = make_float4(B[4], B[5], B[6], B[7]);
  r[2] = make_float4(B[8], s, t, vn[0] + vf[0]);
  r[3] = make_float4(vn[1] + vf[1], vn[2] + vf[2], 0.f, 0.f);
}

template <bool DEFER>
__global__ void __launch_bounds__(PAIR_T, 4) k_pair_member32(xk_pairs32 q, const float* __restrict__ n32,
                                                             xk_contact_params cp, float* __restrict__ rec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // slot = member index
  if (i < q.n_members) member32<DEFER>(q, n32, cp, rec, i);
}

// The deferred (near-parallel) members, grid-stride over the list.
__global__ void __launch_bounds__(PAIR_T) k_pair_member32_deferred(xk_pairs32 q, const float* __restrict__ n32,
                                                                   xk_contact_params cp, float* __restrict__ rec) {
  int32_t* list = q.defer + ((long long)q.cap + DEFER_SLOTS);
  const int cnt = *(volatile const int32_t*)list;
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < cnt; x += gridDim.x * blockDim.x)
    member32<false>(q, n32, cp, rec, list[DEFER_SLOTS + x]);
  if (last_cta_done(list + 1) && threadIdx.x == 0) {
    list[0] = 0;
    list[1] = 0;
  }
}

__global__ void k_active_flags(xk_pairs p, int32_t* __restrict__ flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < p.n) flag[i] = p.status[i] != ST_INACTIVE ? 1 : 0;
}

__global__ void k_jacobian(xk_mesh m, xk_pairs p, const int32_t* __restrict__ off, int32_t* __restrict__ rows,
                           int32_t* __restrict__ cols, double* __restrict__ vals, int32_t* __restrict__ pidx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n || p.status[i] == ST_INACTIVE) return;
  const long long cap = p.cap;
  int r = off[i];
  PairNodes nd = pair_nodes(m, p.ea[i], p.eb[i]);
  double s = p.s[i], t = p.t[i];
  double c[4] = {1.0 - s, s, -(1.0 - t), -t};
  if (pidx) pidx[r] = i;
  for (int k = 0; k < 4; ++k)
    for (int d = 0; d < 3; ++d) {
      long long o = 12LL * r + 3 * k + d;
      rows[o] = r;
      cols[o] = 6 * nd.n[k] + d;
      vals[o] = c[k] * p.normal[d * cap + i];
    }
}

}  // namespace

extern "C" xk_status xk_narrowphase(const xk_mesh* m, xk_pairs* p, const double* u, const xk_contact_params* cp,
                                    int update_active, xk_stream s) {
  if (!m || !p || !u || !cp) return xk_set_error(XK_ERR_ARG, "xk_narrowphase: null argument");
  if (p->n == 0) return XK_OK;
  k_narrow_exact<<<xk_blocks(p->n, PAIR_T), PAIR_T, 0, (cudaStream_t)s>>>(*m, *p, u, cp->g_on, cp->g_off,
                                                                          cp->allow_deactivation, update_active);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_narrowphase_screened(const xk_mesh* m, xk_pairs* p, const double* u, const float* node32,
                                             const xk_contact_params* cp, int32_t* n_exact, xk_stream s) {
  if (!m || !p || !u || !node32 || !cp) return xk_set_error(XK_ERR_ARG, "xk_narrowphase_screened: null argument");
  cudaStream_t st = (cudaStream_t)s;
  if (p->n == 0) {
    if (n_exact) XK_CUDA(cudaMemsetAsync(n_exact, 0, sizeof(int32_t), st));
    return XK_OK;
  }
  int32_t* list = nullptr;
  XK_CUDA(cudaMallocAsync((void**)&list, sizeof(int32_t) * ((size_t)p->n + 1), st));
  xk_status r = XK_OK;
  cudaError_t e = cudaMemsetAsync(list, 0, sizeof(int32_t), st);
  if (e == cudaSuccess) {
    // the thresholds rounded outward to float
    float on_lo = (float)cp->g_on, off_hi = (float)cp->g_off;
    if ((double)on_lo > cp->g_on) on_lo = std::nextafter(on_lo, -INFINITY);
    if ((double)off_hi < cp->g_off) off_hi = std::nextafter(off_hi, INFINITY);
    k_narrow_screen<<<xk_blocks(p->n, PAIR_T), PAIR_T, 0, st>>>(*m, *p, node32, on_lo, off_hi,
                                                               cp->allow_deactivation, list);
    k_narrow_exact_list<<<2 * xk_sm_count(), PAIR_T, 0, st>>>(*m, *p, u, cp->g_on, cp->g_off, cp->allow_deactivation,
                                                              list);
    e = cudaGetLastError();
    if (e == cudaSuccess && n_exact) e = cudaMemcpyAsync(n_exact, list, sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
  }
  if (e != cudaSuccess) r = xk_set_cuda_error(e, __FILE__, __LINE__);
  cudaFreeAsync(list, st);
  return r;
}

extern "C" xk_status xk_pair_step(const xk_mesh* m, xk_pairs* p, const xk_contact_pattern* pat, const double* u,
                                  const double* u_ref, const xk_contact_params* cp, int stages, int precision,
                                  int out_mode, void* rec, xk_stream s) {
  if (!m || !p || !pat || !cp) return xk_set_error(XK_ERR_ARG, "xk_pair_step: null argument");
  if (((stages & XK_STAGE_NARROW) || (stages & XK_STAGE_FRICTION)) && !u)
    return xk_set_error(XK_ERR_ARG, "xk_pair_step: u is required for the narrowphase and friction stages");
  const int all = XK_STAGE_NORMAL | XK_STAGE_FRICTION | XK_STAGE_TANGENT;
  const bool members = !(stages & XK_STAGE_NO_MEMBERS);
  if (members && out_mode == XK_OUT_COMBINED && (stages & all) != all)
    return xk_set_error(XK_ERR_ARG, "xk_pair_step: combined records need the normal, friction and tangent stages");
  if (members && pat->n_members > 0 && !rec) return xk_set_error(XK_ERR_ARG, "xk_pair_step: rec is null");
  if ((long long)pat->n_members + pat->n_others != p->n)
    return xk_set_error(XK_ERR_ARG, "xk_pair_step: pattern was built for another pair table");
  cudaStream_t st = (cudaStream_t)s;
  if ((stages & XK_STAGE_NARROW) && !(stages & XK_STAGE_NO_OTHERS) && pat->n_others > 0) {
    const int nb = xk_blocks(pat->n_others, PAIR_T);
    if (precision == XK_FP64)
      k_pair_other<XK_FP64><<<nb, PAIR_T, 0, st>>>(*m, *p, pat->others, pat->n_others, u);
    else if (precision == XK_MIXED)
      k_pair_other<XK_MIXED><<<nb, PAIR_T, 0, st>>>(*m, *p, pat->others, pat->n_others, u);
    else
      return xk_set_error(XK_ERR_ARG, "xk_pair_step: precision");
    XK_CHECK_LAUNCH();
  }
  if (pat->n_members == 0 || (stages & XK_STAGE_NO_MEMBERS)) return XK_OK;
  const int nb = xk_blocks(pat->n_members, PAIR_T);
  const long long rs = out_mode == XK_OUT_COMBINED ? XK_REC_STRIDE_COMBINED : XK_REC_STRIDE_SPLIT;
  const bool coat = m->core_radii && p->coat_cc;
#define XK_MEMBER_LAUNCH(PP, OO, CC, TT)                                                                        \
  k_pair_member<PP, OO, CC><<<nb, PAIR_T, 0, st>>>(*m, *p, pat->members, pat->member_nodes, pat->n_members, u,  \
                                                   u_ref, *cp, stages, (TT*)rec, rs)
  if (precision == XK_FP64) {
    if (out_mode == XK_OUT_COMBINED) {
      if (coat) XK_MEMBER_LAUNCH(XK_FP64, XK_OUT_COMBINED, true, double);
      else XK_MEMBER_LAUNCH(XK_FP64, XK_OUT_COMBINED, false, double);
    } else {
      XK_MEMBER_LAUNCH(XK_FP64, XK_OUT_SPLIT, false, double);
    }
  } else if (precision == XK_MIXED) {
    if (out_mode == XK_OUT_COMBINED) {
      if (coat) XK_MEMBER_LAUNCH(XK_MIXED, XK_OUT_COMBINED, true, float);
      else XK_MEMBER_LAUNCH(XK_MIXED, XK_OUT_COMBINED, false, float);
    } else {
      XK_MEMBER_LAUNCH(XK_MIXED, XK_OUT_SPLIT, false, float);
    }
  } else {
    return xk_set_error(XK_ERR_ARG, "xk_pair_step: precision");
  }
#undef XK_MEMBER_LAUNCH
  XK_CHECK_LAUNCH();
  return XK_OK;
}

namespace {
// Smooth (softplus) normal law, element-wise: _evaluate_smooth_normal_force_vectorized
// (contact/penalty/law_normal.py:129-149); exp and log1p are the CUDA double functions.
__global__ void k_softplus_law(long long n, const double* __restrict__ g, const double* __restrict__ lam, double k,
                               double delta, double* __restrict__ p, double* __restrict__ dp) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = k > 0.0 ? xadd(-g[i], lam ? xdiv(lam[i], k) : 0.0) : -g[i];
  const double z = xdiv(x, delta);
  const double ez = exp(z < -30.0 ? -30.0 : (z > 30.0 ? 30.0 : z));
  const double sp = z > 30.0 ? x : (z < -30.0 ? 0.0 : xmul(delta, log1p(ez)));
  const double sig = z > 30.0 ? 1.0 : (z < -30.0 ? 0.0 : xdiv(ez, xadd(1.0, ez)));
  p[i] = xmul(k, sp);
  dp[i] = xmul(-k, sig);
}
}  // namespace

namespace {
// _auto_select_n_gauss (geometry/_compute.py:264-291) at X + u for one pair
__global__ void k_gauss_points(xk_mesh m, xk_pairs p, const double* __restrict__ u, int default_n,
                               int8_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int ea = p.ea[i], eb = p.eb[i];
  const int nd[4] = {m.conn[2 * ea], m.conn[2 * ea + 1], m.conn[2 * eb], m.conn[2 * eb + 1]};
  double x[4][3];
  for (int k = 0; k < 4; ++k)
    for (int c = 0; c < 3; ++c) x[k][c] = u ? xadd(m.X[3LL * nd[k] + c], u[6LL * nd[k] + c]) : m.X[3LL * nd[k] + c];
  double dA[3], dB[3];
  for (int c = 0; c < 3; ++c) {
    dA[c] = xsub(x[1][c], x[0][c]);
    dB[c] = xsub(x[3][c], x[2][c]);
  }
  const double lenA = xsqrt(xdot_seq(dA, dA)), lenB = xsqrt(xdot_seq(dB, dB));
  int n = default_n;
  if (!(lenA < 1e-30 || lenB < 1e-30)) {
    const double c = fabs(xdiv(xdot_seq(dA, dB), xmul(lenA, lenB)));
    n = c < 0.866 ? 2 : (c < 0.985 ? 3 : 5);
  }
  out[i] = (int8_t)n;
}
}  // namespace

extern "C" xk_status xk_pair_gauss_points(const xk_mesh* m, const xk_pairs* p, const double* u, int32_t default_n,
                                          int8_t* out, xk_stream s) {
  if (!m || !p || (p->n > 0 && !out)) return xk_set_error(XK_ERR_ARG, "xk_pair_gauss_points: null argument");
  if (p->n == 0) return XK_OK;
  k_gauss_points<<<xk_blocks(p->n, 256), 256, 0, (cudaStream_t)s>>>(*m, *p, u, default_n, out);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_softplus_normal_law(int64_t n, const double* gaps, const double* lambdas, double k_pen,
                                            double delta, double* p_n, double* dp_dg, xk_stream s) {
  if (n < 0 || (n > 0 && (!gaps || !p_n || !dp_dg)) || !(delta > 0.0))
    return xk_set_error(XK_ERR_ARG, "xk_softplus_normal_law: bad arguments");
  if (n == 0) return XK_OK;
  k_softplus_law<<<xk_blocks(n, 256), 256, 0, (cudaStream_t)s>>>(n, gaps, lambdas, k_pen, delta, p_n, dp_dg);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_constraint_jacobian(const xk_mesh* m, const xk_pairs* p, int32_t* rows, int32_t* cols,
                                            double* vals, int32_t* pair_index, int64_t cap, int64_t* n_rows,
                                            xk_stream s) {
  if (!m || !p || !n_rows) return xk_set_error(XK_ERR_ARG, "xk_constraint_jacobian: null argument");
  cudaStream_t st = (cudaStream_t)s;
  *n_rows = 0;
  if (p->n == 0) return XK_OK;
  int32_t* flag = nullptr;
  int64_t* tot = nullptr;
  XK_CUDA(cudaMallocAsync((void**)&flag, sizeof(int32_t) * p->n, st));
  XK_CUDA(cudaMallocAsync((void**)&tot, sizeof(int64_t), st));
  k_active_flags<<<xk_blocks(p->n, 256), 256, 0, st>>>(*p, flag);
  xk_status r = xk_exclusive_scan_i32(flag, flag, p->n, tot, st);
  int64_t h = 0;
  if (r == XK_OK) {
    cudaError_t e = cudaMemcpyAsync(&h, tot, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) r = xk_set_cuda_error(e, __FILE__, __LINE__);
  }
  if (r == XK_OK) {
    *n_rows = h;
    if (h > cap) {
      r = xk_set_error(XK_ERR_CAPACITY, "xk_constraint_jacobian: capacity below the number of active pairs");
    } else if (h > 0) {
      k_jacobian<<<xk_blocks(p->n, 256), 256, 0, st>>>(*m, *p, flag, rows, cols, vals, pair_index);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) r = xk_set_cuda_error(e, __FILE__, __LINE__);
    }
  }
  cudaFreeAsync(flag, st);
  cudaFreeAsync(tot, st);
  return r;
}

// ---------------------------------------------------------------------------
// xk_constraint_jacobian_noalloc: the same kernels with their scratch in one
// static device array instead of stream-ordered allocations, for callers that
// may not allocate device memory while they run (a host that has handed all
// of the device's memory to its own pool, or a loop that must not go through
// the allocator).  Layout in int64 words: [0, 32) the active-pair count,
// [32, 32 + JNA_TILES) the scan's block sums, then one int32 flag/offset per
// pair.  Every word is written before it is read, so nothing has to start at
// zero.  The array is shared by every call on a device: calls that overlap
// (two streams or two host threads) race on it and must be serialised.
namespace {
constexpr long long JNA_MAX_PAIRS = XK_JACOBIAN_NOALLOC_MAX_PAIRS;
constexpr long long JNA_TILES = 1024;  // block sums for up to 2,097,152 scanned elements
constexpr long long JNA_WORDS = 32 + JNA_TILES + JNA_MAX_PAIRS / 2;
static_assert(JNA_MAX_PAIRS % 2 == 0, "flags are packed two per word");

static __device__ __align__(256) int64_t g_jna_scratch[JNA_WORDS];

// Id of the calling thread's current context (CUDA 12's cuCtxGetId, reached
// through the runtime's driver entry points so that the library needs no
// libcuda at link time); false when there is no current context yet or the
// driver does not offer the calls.
using PfnCtxGetCurrent = CUresult (*)(CUcontext*);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);
bool current_context_id(unsigned long long* id) {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PfnCtxGetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PfnCtxGetId>(f);
  });
  CUcontext c = nullptr;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c) return false;
  return get_id(c, id) == CUDA_SUCCESS;
}

// Address of the scratch array in the current context.  The look-up loads this
// module's device globals into the context, so the first call in a context is
// the set-up call; make it before any work that must not see one.  The address
// is cached per device ordinal together with the id of the context it belongs
// to: a context created later on that device (after cudaDeviceReset, or a
// non-primary context) has another id and is looked up again.
struct JnaCache {
  unsigned long long ctx = 0;
  int64_t* ptr = nullptr;
};
std::mutex g_jna_mutex;
JnaCache g_jna_cache[64];

xk_status jna_scratch(int64_t** out) {
  int dev = 0;
  XK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return xk_set_error(XK_ERR_ARG, "device ordinal out of range");
  unsigned long long cid = 0;
  bool have = current_context_id(&cid);
  if (have) {
    std::lock_guard<std::mutex> lock(g_jna_mutex);
    if (g_jna_cache[dev].ptr && g_jna_cache[dev].ctx == cid) {
      *out = g_jna_cache[dev].ptr;
      return XK_OK;
    }
  }
  int64_t* p = nullptr;
  XK_CUDA(cudaGetSymbolAddress((void**)&p, g_jna_scratch));
  if (!have) have = current_context_id(&cid);  // the look-up made the primary context current
  if (have) {
    std::lock_guard<std::mutex> lock(g_jna_mutex);
    g_jna_cache[dev].ctx = cid;
    g_jna_cache[dev].ptr = p;
  }
  *out = p;
  return XK_OK;
}
}  // namespace

extern "C" xk_status xk_constraint_jacobian_noalloc(const xk_mesh* m, const xk_pairs* p, int32_t* rows,
                                                    int32_t* cols, double* vals, int32_t* pair_index, int64_t cap,
                                                    int64_t* n_rows, xk_stream s) {
  if (!m || !p || !n_rows) return xk_set_error(XK_ERR_ARG, "xk_constraint_jacobian_noalloc: null argument");
  *n_rows = 0;
  if (p->n < 0 || (long long)p->n > JNA_MAX_PAIRS)
    return xk_set_error(XK_ERR_ARG,
                        "xk_constraint_jacobian_noalloc: pair table larger than XK_JACOBIAN_NOALLOC_MAX_PAIRS "
                        "(1048576); use xk_constraint_jacobian");
  if (xk_scan_tiles(p->n) > JNA_TILES) return xk_set_error(XK_ERR_ARG, "xk_constraint_jacobian_noalloc: scan tiles");
  int64_t* scratch = nullptr;
  xk_status r = jna_scratch(&scratch);
  if (r != XK_OK) return r;
  if (p->n == 0) return XK_OK;
  cudaStream_t st = (cudaStream_t)s;
  int64_t* tot = scratch;
  int64_t* bsum = scratch + 32;
  int32_t* flag = (int32_t*)(scratch + 32 + JNA_TILES);
  k_active_flags<<<xk_blocks(p->n, 256), 256, 0, st>>>(*p, flag);
  XK_CHECK_LAUNCH();
  r = xk_exclusive_scan_i32_scratch(flag, flag, p->n, tot, bsum, JNA_TILES, st);
  if (r != XK_OK) return r;
  int64_t h = 0;
  XK_CUDA(cudaMemcpyAsync(&h, tot, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  XK_CUDA(cudaStreamSynchronize(st));
  *n_rows = h;
  if (h > cap) return xk_set_error(XK_ERR_CAPACITY, "xk_constraint_jacobian_noalloc: capacity below the number "
                                                    "of active pairs");
  if (h > 0) {
    k_jacobian<<<xk_blocks(p->n, 256), 256, 0, st>>>(*m, *p, flag, rows, cols, vals, pair_index);
    XK_CHECK_LAUNCH();
  }
  return XK_OK;
}

extern "C" xk_status xk_nodes_prepare(const xk_mesh* m, const double* u, const double* u_ref, float* node32,
                                      xk_stream s) {
  if (!m || !u || !node32) return xk_set_error(XK_ERR_ARG, "xk_nodes_prepare: null argument");
  if (m->n_nodes == 0) return XK_OK;
  if (((uintptr_t)node32 & 15) != 0) return xk_set_error(XK_ERR_ARG, "xk_nodes_prepare: node32 must be 16-byte aligned");
  const bool vec = ((uintptr_t)u & 15) == 0 && ((uintptr_t)u_ref & 15) == 0;
  if (vec)
    k_nodes_prepare<true><<<xk_blocks(m->n_nodes, 128), 128, 0, (cudaStream_t)s>>>(*m, u, u_ref, node32);
  else
    k_nodes_prepare<false><<<xk_blocks(m->n_nodes, 128), 128, 0, (cudaStream_t)s>>>(*m, u, u_ref, node32);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_pairs_to32(const xk_mesh* m, const xk_pairs* p, const xk_contact_pattern* pat, xk_pairs32* q,
                                   xk_stream s) {
  if (!m || !p || !pat || !q) return xk_set_error(XK_ERR_ARG, "xk_pairs_to32: null argument");
  if ((long long)pat->n_members + pat->n_others != p->n)
    return xk_set_error(XK_ERR_ARG, "xk_pairs_to32: the pattern was built for another pair table");
  if (q->cap < p->n) return xk_set_error(XK_ERR_CAPACITY, "xk_pairs_to32: float table capacity below n");
  q->n = p->n;
  q->n_members = pat->n_members;
  if (p->n == 0) return XK_OK;
  k_pairs_to32<<<xk_blocks(p->n, 256), 256, 0, (cudaStream_t)s>>>(*m, *p, *pat, *q);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_pairs_from32(const xk_pairs32* q, xk_pairs* p, xk_stream s) {
  if (!q || !p) return xk_set_error(XK_ERR_ARG, "xk_pairs_from32: null argument");
  if (q->n != p->n) return xk_set_error(XK_ERR_ARG, "xk_pairs_from32: table sizes differ");
  if (q->n == 0) return XK_OK;
  if (q->slot)
    k_pairs_from32<true><<<xk_blocks(q->n, 256), 256, 0, (cudaStream_t)s>>>(*q, *p);
  else
    k_pairs_from32<false><<<xk_blocks(q->n, 256), 256, 0, (cudaStream_t)s>>>(*q, *p);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_pair_step32(xk_pairs32* q, const float* node32, const xk_contact_params* cp, float* rec,
                                    int parts, xk_stream s) {
  if (!q || !node32 || !cp) return xk_set_error(XK_ERR_ARG, "xk_pair_step32: null argument");
  if (((uintptr_t)node32 & 31) != 0 || ((uintptr_t)rec & 15) != 0)
    return xk_set_error(XK_ERR_ARG, "xk_pair_step32: node32 must be 32-byte and rec 16-byte aligned");
  if ((parts & XK_PAIRS_MEMBERS) && q->n_members > 0 && !rec)
    return xk_set_error(XK_ERR_ARG, "xk_pair_step32: rec is null");
  cudaStream_t st = (cudaStream_t)s;
  const int n_o = q->n - q->n_members;
  // the CTA size of the common kernels: a launch-shape choice only (each thread owns one slot)
  const int bs = (q->block >= 32 && q->block <= PAIR_T && q->block % 32 == 0) ? q->block : PAIR_T;
  if ((parts & XK_PAIRS_OTHERS) && n_o > 0) {
    if (q->defer) {
      k_pair_other32<true><<<xk_blocks(n_o, bs), bs, 0, st>>>(*q, node32);
      k_pair_other32_deferred<<<152, PAIR_T, 0, st>>>(*q, node32);
    } else {
      k_pair_other32<false><<<xk_blocks(n_o, bs), bs, 0, st>>>(*q, node32);
    }
  }
  if ((parts & XK_PAIRS_MEMBERS) && q->n_members > 0) {
    if (q->defer) {
      k_pair_member32<true><<<xk_blocks(q->n_members, bs), bs, 0, st>>>(*q, node32, *cp, rec);
      k_pair_member32_deferred<<<152, PAIR_T, 0, st>>>(*q, node32, *cp, rec);
    } else {
      k_pair_member32<false><<<xk_blocks(q->n_members, bs), bs, 0, st>>>(*q, node32, *cp, rec);
    }
  }
  XK_CHECK_LAUNCH();
  return XK_OK;
}
