// Coated-wire contact (Kelvin-Voigt coating with Coulomb friction on the
// coating surface): KelvinVoigtCoatingProcess (xkep_cae/contact/coating/
// strategy.py:80-400) and the coating branch of UpdateGeometryProcess
// (xkep_cae/contact/_manager_process.py:351-360, 386-396, 475-494).
//
// The geometry runs the exact narrowphase on the core radii (gap = dist -
// (core_a + core_b)); xk_coating_geometry then forms the coating compression
// cc = max(0, coat_total - gap) and, unless the active set is frozen, applies
// the hysteresis with the coating term.  The forces and tangents are written
// as split member records, as the contact pair kernels write theirs: the
// force on a pair's local node k is c_k v and its tangent block (k, l) is
// c_k c_l B, c = [1-s, s, -(1-t), -t].  The elastic / viscous coating force
// is the normal part of the record (v_n, B_n), the coating friction its
// friction part (v_f, B_f).
#include <math.h>

#include "xk_common.cuh"

namespace {

constexpr uint8_t ST_INACTIVE = 0, ST_ACTIVE = 1;

__global__ void k_coating_geometry(xk_pairs p, const double* __restrict__ coat_total, double g_on, double g_off,
                                   int allow_deact, int update_active, double* __restrict__ cc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const double gap = p.gap[i];
  const double c = fmax(0.0, xsub(coat_total[i], gap));  // np.maximum(0.0, coat_total - gap_core)
  cc[i] = c;
  if (update_active) {  // _update_active_set_state with the coating term
    const bool coat_active = c > 0.0;
    const uint8_t st = p.status[i];
    if (st == ST_INACTIVE) {
      if (gap <= g_on || coat_active) p.status[i] = ST_ACTIVE;
    } else if (allow_deact && gap >= g_off && !coat_active) {
      p.status[i] = ST_INACTIVE;
    }
  }
}

XK_D void load3d(const double* base, long long cap, int i, double* v) {
  v[0] = base[i];
  v[1] = base[cap + i];
  v[2] = base[2 * cap + i];
}

// _tangent_2x2_core (contact/friction/law_friction.py:126-153)
XK_D void tangent2x2(double k_t, double p_n, double mu, double z0, double z1, double qtn, bool stick, double* D) {
  D[0] = D[1] = D[2] = D[3] = 0.0;
  if (p_n <= 0.0 || mu <= 0.0) return;
  const double zn = sqrt(xadd(xmul(z0, z0), xmul(z1, z1)));
  if (stick || zn < 1e-30 || qtn < 1e-30) {
    D[0] = k_t;
    D[3] = k_t;
    return;
  }
  const double h0 = z0 / zn, h1 = z1 / zn, ratio = (mu * p_n) / qtn;
  D[0] = ratio * k_t * (1.0 - h0 * h0);
  D[1] = ratio * k_t * (0.0 - h0 * h1);
  D[2] = D[1];
  D[3] = ratio * k_t * (1.0 - h1 * h1);
}

__global__ void k_coating_step(xk_pairs p, const int32_t* __restrict__ members, const int32_t* __restrict__ mnodes,
                               int n_m, xk_coating_state cs, const double* __restrict__ u,
                               const double* __restrict__ u_ref, xk_coating_params cp, int stages,
                               double* __restrict__ rec) {
  const int mi = blockIdx.x * blockDim.x + threadIdx.x;
  if (mi >= n_m) return;
  const int i = members[mi];
  const long long cap = p.cap;
  const double s = p.s[i], t = p.t[i];
  double n[3], t1[3], t2[3];
  load3d(p.normal, cap, i, n);
  load3d(p.t1, cap, i, t1);
  load3d(p.t2, cap, i, t2);
  const double cc = cs.cc[i];
  double* r = rec + (long long)mi * XK_REC_STRIDE_SPLIT;  // (s, t, v_n, v_f, B_n, B_f)
  r[0] = s;
  r[1] = t;
  const bool visc = cp.damping > 0.0 && cp.dt > 0.0;
  if (stages & XK_COAT_FORCE) {  // forces (strategy.py:97-143)
    double vn[3] = {0.0, 0.0, 0.0};
    const double prev = cs.cc_prev[i];
    if (!(cc <= 0.0 && prev <= 0.0)) {
      double f = cp.stiffness * cc;
      if (visc) f += cp.damping * ((cc - prev) / cp.dt);
      if (!(fabs(f) < 1e-30))
        for (int k = 0; k < 3; ++k) vn[k] = -f * n[k];
    }
    for (int k = 0; k < 3; ++k) r[2 + k] = vn[k];
  }
  if (stages & XK_COAT_TANGENT) {  // stiffness (strategy.py:145-196): k_eff n n^T
    const double k_eff = visc ? cp.stiffness + cp.damping / cp.dt : cp.stiffness;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) r[8 + 3 * a + b] = cc > 1e-15 ? k_eff * n[a] * n[b] : 0.0;
  }
  const double k_t = cp.stiffness * cp.k_t_ratio;
  if (stages & XK_COAT_FRICTION) {  // friction_forces (strategy.py:198-288)
    double vf[3] = {0.0, 0.0, 0.0};
    if (cc <= 0.0) {  // no coating contact: the friction history is reset
      cs.z_t[i] = 0.0;
      cs.z_t[cap + i] = 0.0;
      cs.stick[i] = 1;
      cs.q_trial_norm[i] = 0.0;
      cs.dissipation[i] = 0.0;
    } else {
      const double p_n = cp.stiffness * cc;
      const int nd[4] = {mnodes[4LL * mi], mnodes[4LL * mi + 1], mnodes[4LL * mi + 2], mnodes[4LL * mi + 3]};
      double du[4][3];
      for (int k = 0; k < 4; ++k)
        for (int c = 0; c < 3; ++c) {
          const long long dof = 6LL * nd[k] + c;
          du[k][c] = u_ref ? u[dof] - u_ref[dof] : u[dof];
        }
      double rel[3];
      for (int c = 0; c < 3; ++c)
        rel[c] = ((1.0 - t) * du[2][c] + t * du[3][c]) - ((1.0 - s) * du[0][c] + s * du[1][c]);
      const double d0 = xdot_seq(rel, t1), d1 = xdot_seq(rel, t2);
      double q0 = 0.0, q1 = 0.0, qtn = 0.0, diss = 0.0;
      bool stick = true;
      if (p_n > 0.0 && cp.mu > 0.0) {  // _return_mapping_core (law_friction.py:89-123)
        const double tr0 = cs.z_t[i] + k_t * d0, tr1 = cs.z_t[cap + i] + k_t * d1;
        qtn = sqrt(tr0 * tr0 + tr1 * tr1);
        const double fy = cp.mu * p_n;
        if (qtn <= fy) {
          q0 = tr0;
          q1 = tr1;
        } else {
          q0 = fy * tr0 / qtn;
          q1 = fy * tr1 / qtn;
          stick = false;
        }
        diss = q0 * d0 + q1 * d1;
      }
      cs.z_t[i] = q0;
      cs.z_t[cap + i] = q1;
      cs.stick[i] = stick ? 1 : 0;
      cs.q_trial_norm[i] = qtn;
      cs.dissipation[i] = diss;
      for (int k = 0; k < 3; ++k) vf[k] = -(q0 * t1[k] + q1 * t2[k]);
    }
    for (int k = 0; k < 3; ++k) r[5 + k] = vf[k];
  }
  if (stages & XK_COAT_FRICTION_TANGENT) {  // friction_stiffness (strategy.py:290-370): T D T^T
    double D[4] = {0.0, 0.0, 0.0, 0.0};
    if (cc > 0.0)
      tangent2x2(k_t, cp.stiffness * cc, cp.mu, cs.z_t[i], cs.z_t[cap + i], cs.q_trial_norm[i], cs.stick[i] != 0, D);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        r[17 + 3 * a + b] = (t1[a] * D[0] + t2[a] * D[2]) * t1[b] + (t1[a] * D[1] + t2[a] * D[3]) * t2[b];
  }
}

}  // namespace

extern "C" xk_status xk_coating_geometry(xk_pairs* p, const double* coat_total, const xk_contact_params* cp,
                                         int update_active, double* cc, xk_stream s) {
  if (!p || !cp || (p->n > 0 && (!coat_total || !cc))) return xk_set_error(XK_ERR_ARG, "xk_coating_geometry: null argument");
  if (p->n == 0) return XK_OK;
  k_coating_geometry<<<xk_blocks(p->n, 256), 256, 0, (cudaStream_t)s>>>(*p, coat_total, cp->g_on, cp->g_off,
                                                                          cp->allow_deactivation, update_active, cc);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_coating_step(const xk_pairs* p, const xk_contact_pattern* pat, xk_coating_state* cs,
                                     const double* u, const double* u_ref, const xk_coating_params* cp, int stages,
                                     double* rec, xk_stream s) {
  if (!p || !pat || !cs || !cp) return xk_set_error(XK_ERR_ARG, "xk_coating_step: null argument");
  if (pat->n_members == 0) return XK_OK;
  if (!rec || !cs->cc || ((stages & XK_COAT_FORCE) && !cs->cc_prev) ||
      ((stages & (XK_COAT_FRICTION | XK_COAT_FRICTION_TANGENT)) &&
       (!cs->z_t || !cs->stick || !cs->q_trial_norm || !cs->dissipation)) || ((stages & XK_COAT_FRICTION) && !u))
    return xk_set_error(XK_ERR_ARG, "xk_coating_step: missing array for the selected stages");
  k_coating_step<<<xk_blocks(pat->n_members, 128), 128, 0, (cudaStream_t)s>>>(*p, pat->members, pat->member_nodes,
                                                                              pat->n_members, *cs, u, u_ref, *cp,
                                                                              stages, rec);
  XK_CHECK_LAUNCH();
  return XK_OK;
}
