// Generalized-alpha time integration on the device (lumped mass, no damping):
// predictor, corrector, effective residual and the mass term of the effective
// stiffness, as GeneralizedAlphaProcess (xkep_cae/time_integration/strategy.py:96-232).
// Element-wise FP64 in the reference's operation order (no contraction).
#include "xk_common.cuh"

namespace {

// u_pred = (u + dt v) + c2 a, v_pred = v + c3 a with c2 = 0.5 dt^2 (1 - 2 beta), c3 = dt (1 - gamma)
__global__ void k_ga_predict(long long n, const double* __restrict__ u, const double* __restrict__ vel,
                             const double* __restrict__ acc, double* __restrict__ vel_old,
                             double* __restrict__ acc_old, double* __restrict__ u_pred, double* __restrict__ v_pred,
                             double dt, double c2, double c3) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = acc[i], v = vel[i];
  acc_old[i] = a;
  vel_old[i] = v;
  u_pred[i] = xadd(xadd(u[i], xmul(dt, v)), xmul(c2, a));
  v_pred[i] = xadd(v, xmul(c3, a));
}

// a = c0 (u - u_pred), v = v_pred + (dt gamma) a
__global__ void k_ga_correct(long long n, const double* __restrict__ u, const double* __restrict__ u_pred,
                             const double* __restrict__ v_pred, double* __restrict__ acc, double* __restrict__ vel,
                             double c0, double dg) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = xmul(c0, xsub(u[i], u_pred[i]));
  acc[i] = a;
  vel[i] = xadd(v_pred[i], xmul(dg, a));
}

// out = R + m ((1 - alpha_m) a + alpha_m a_old)
__global__ void k_ga_residual(long long n, const double* __restrict__ R, const double* __restrict__ m,
                              const double* __restrict__ acc, const double* __restrict__ acc_old, double oam,
                              double am, double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = xadd(R[i], xmul(m[i], xadd(xmul(oam, acc[i]), xmul(am, acc_old[i]))));
}

template <typename T>
__global__ void k_add_diag(long long n, const int64_t* __restrict__ idx, const double* __restrict__ m, double c,
                           T* __restrict__ K) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || idx[i] < 0) return;  // a node without elements has no diagonal block
  K[idx[i]] += (T)xmul(c, m[i]);
}

}  // namespace

extern "C" xk_status xk_genalpha_predict(int64_t n, const double* u, const double* vel, const double* acc,
                                         double* vel_old, double* acc_old, double* u_pred, double* v_pred, double dt,
                                         double beta, double gamma, xk_stream s) {
  if (n < 0 || (n > 0 && (!u || !vel || !acc || !vel_old || !acc_old || !u_pred || !v_pred)))
    return xk_set_error(XK_ERR_ARG, "xk_genalpha_predict: bad arguments");
  if (n == 0) return XK_OK;
  const double c2 = (0.5 * (dt * dt)) * (1.0 - 2.0 * beta), c3 = dt * (1.0 - gamma);
  k_ga_predict<<<xk_blocks(n, 256), 256, 0, (cudaStream_t)s>>>(n, u, vel, acc, vel_old, acc_old, u_pred, v_pred, dt,
                                                               c2, c3);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_genalpha_correct(int64_t n, const double* u, const double* u_pred, const double* v_pred,
                                         double* acc, double* vel, double dt, double beta, double gamma,
                                         xk_stream s) {
  if (n < 0 || (n > 0 && (!u || !u_pred || !v_pred || !acc || !vel)))
    return xk_set_error(XK_ERR_ARG, "xk_genalpha_correct: bad arguments");
  if (n == 0 || dt < 1e-30) return XK_OK;
  const double c0 = 1.0 / (beta * (dt * dt)), dg = dt * gamma;
  k_ga_correct<<<xk_blocks(n, 256), 256, 0, (cudaStream_t)s>>>(n, u, u_pred, v_pred, acc, vel, c0, dg);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_genalpha_residual(int64_t n, const double* R, const double* m, const double* acc,
                                          const double* acc_old, double alpha_m, double* out, xk_stream s) {
  if (n < 0 || (n > 0 && (!R || !m || !acc || !acc_old || !out)))
    return xk_set_error(XK_ERR_ARG, "xk_genalpha_residual: bad arguments");
  if (n == 0) return XK_OK;
  k_ga_residual<<<xk_blocks(n, 256), 256, 0, (cudaStream_t)s>>>(n, R, m, acc, acc_old, 1.0 - alpha_m, alpha_m, out);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_add_diagonal(int64_t n, const int64_t* idx, const double* m, double c, int precision,
                                     void* K, xk_stream s) {
  if (n < 0 || (n > 0 && (!idx || !m || !K))) return xk_set_error(XK_ERR_ARG, "xk_add_diagonal: bad arguments");
  if (n == 0) return XK_OK;
  if (precision == XK_FP64)
    k_add_diag<double><<<xk_blocks(n, 256), 256, 0, (cudaStream_t)s>>>(n, idx, m, c, (double*)K);
  else if (precision == XK_MIXED)
    k_add_diag<float><<<xk_blocks(n, 256), 256, 0, (cudaStream_t)s>>>(n, idx, m, c, (float*)K);
  else
    return xk_set_error(XK_ERR_ARG, "xk_add_diagonal: precision");
  XK_CHECK_LAUNCH();
  return XK_OK;
}
