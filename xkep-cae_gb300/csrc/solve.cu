// The Newton step's linear system on the device: LinearSolveProcess
// (xkep_cae/contact/solver/_newton_steps.py:338-366) solves K du = -R with the
// Dirichlet DOFs' rows and columns replaced by the identity by a sparse direct
// factorisation on the host.  Here the system stays where the assembly left it,
// K = K_beam (6x6 blocks over the nodes) + K_c (3x3 blocks over the nodes'
// translational DOFs), and is solved by BiCGStab with a block-Jacobi
// preconditioner (each node's 6x6 diagonal block, inverted once per matrix).
// Every reduction is a fixed-order two-pass sum (block partial sums in a fixed
// grid, then one block), so a solve gives the same bits run after run; the
// iteration's scalars stay in device memory, so a solve issues no host
// synchronisation until its convergence checks.
#include <math.h>

#include "xk_common.cuh"

namespace {

constexpr int SV_T = 256;
constexpr int SV_BLOCKS = 304;  // 2 x 152 SMs: the fixed grid of the two-pass reductions

template <typename T>
__global__ void k_spmv(xk_system A, const double* __restrict__ x, double* __restrict__ y) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= 6LL * A.n_nodes) return;
  const int v = (int)(g / 6), d = (int)(g % 6);
  if (A.fixed && A.fixed[g]) {  // Dirichlet row: identity
    y[g] = x[g];
    return;
  }
  const T* kb = (const T*)A.kb_vals;
  double acc = 0.0;
  // the stored blocks (u, v), u < v, transposed: row v's blocks left of the diagonal
  for (int q = A.kb_low_ptr[v]; q < A.kb_low_ptr[v + 1]; ++q) {
    const int b = A.kb_low_blk[q];
    const int u = A.kb_blk_row[b];
    const T* blk = kb + 36LL * b + d;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const long long col = 6LL * u + j;
      if (!(A.fixed && A.fixed[col])) acc = fma((double)blk[6 * j], x[col], acc);
    }
  }
  for (int b = A.kb_row_ptr[v]; b < A.kb_row_ptr[v + 1]; ++b) {
    const int w = A.kb_col[b];
    const T* blk = kb + 36LL * b + 6 * d;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const long long col = 6LL * w + j;
      if (!(A.fixed && A.fixed[col])) acc = fma((double)blk[j], x[col], acc);
    }
  }
  if (d < 3 && A.kc_vals) {
    const T* kc = (const T*)A.kc_vals;
    // the stored blocks (u, v), u < v, are also the blocks (v, u): row v's entries left of the diagonal
    for (int q = A.kc_low_ptr[v]; q < A.kc_low_ptr[v + 1]; ++q) {
      const int b = A.kc_low_blk[q];
      const int u = A.kc_blk_row[b];
      const T* blk = kc + 9LL * b + 3 * d;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const long long col = 6LL * u + j;
        if (!(A.fixed && A.fixed[col])) acc = fma((double)blk[j], x[col], acc);
      }
    }
    for (int b = A.kc_row_ptr[v]; b < A.kc_row_ptr[v + 1]; ++b) {
      const int w = A.kc_col[b];
      const T* blk = kc + 9LL * b + 3 * d;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const long long col = 6LL * w + j;
        if (!(A.fixed && A.fixed[col])) acc = fma((double)blk[j], x[col], acc);
      }
    }
  }
  y[g] = acc;
}

// inverse of each node's 6x6 diagonal block (K_beam's, plus K_c's translational one), Dirichlet DOFs
// as identity rows and columns; Gauss-Jordan with partial pivoting in double
template <typename T>
__global__ void k_block_jacobi(xk_system A, double* __restrict__ dinv) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.n_nodes) return;
  double M[6][12];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 12; ++j) M[i][j] = (j - 6 == i) ? 1.0 : 0.0;
  const T* kb = (const T*)A.kb_vals;
  for (int b = A.kb_row_ptr[v]; b < A.kb_row_ptr[v + 1]; ++b)
    if (A.kb_col[b] == v)
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) M[i][j] += (double)kb[36LL * b + 6 * i + j];
  if (A.kc_vals) {
    const T* kc = (const T*)A.kc_vals;
    for (int b = A.kc_row_ptr[v]; b < A.kc_row_ptr[v + 1]; ++b)
      if (A.kc_col[b] == v)
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) M[i][j] += (double)kc[9LL * b + 3 * i + j];
  }
  if (A.fixed)
    for (int i = 0; i < 6; ++i)
      if (A.fixed[6LL * v + i])
        for (int j = 0; j < 6; ++j) {
          M[i][j] = (i == j) ? 1.0 : 0.0;
          M[j][i] = (i == j) ? 1.0 : 0.0;
        }
  for (int c = 0; c < 6; ++c) {
    int piv = c;
    for (int r = c + 1; r < 6; ++r)
      if (fabs(M[r][c]) > fabs(M[piv][c])) piv = r;
    if (piv != c)
      for (int j = 0; j < 12; ++j) {
        const double t = M[c][j];
        M[c][j] = M[piv][j];
        M[piv][j] = t;
      }
    const double p = M[c][c];
    const double ip = fabs(p) > 0.0 ? 1.0 / p : 0.0;  // a singular block leaves that part unpreconditioned
    for (int j = 0; j < 12; ++j) M[c][j] *= ip;
    for (int r = 0; r < 6; ++r)
      if (r != c) {
        const double f = M[r][c];
        for (int j = 0; j < 12; ++j) M[r][j] -= f * M[c][j];
      }
  }
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) dinv[36LL * v + 6 * i + j] = M[i][6 + j];
}

__global__ void k_apply_block_jacobi(int n_nodes, const double* __restrict__ dinv, const double* __restrict__ r,
                                     double* __restrict__ z) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= 6LL * n_nodes) return;
  const int v = (int)(g / 6), d = (int)(g % 6);
  const double* D = dinv + 36LL * v + 6 * d;
  double acc = 0.0;
#pragma unroll
  for (int j = 0; j < 6; ++j) acc = fma(D[j], r[6LL * v + j], acc);
  z[g] = acc;
}

// block partial sums of up to two dot products: part[2 b + k] = sum over the block's grid-stride share
__global__ void k_dot2(long long n, const double* __restrict__ a0, const double* __restrict__ b0,
                       const double* __restrict__ a1, const double* __restrict__ b1, double* __restrict__ part) {
  __shared__ double red[2][SV_T];
  double s0 = 0.0, s1 = 0.0;
  for (long long i = (long long)blockIdx.x * SV_T + threadIdx.x; i < n; i += (long long)SV_BLOCKS * SV_T) {
    s0 = fma(a0[i], b0[i], s0);
    if (a1) s1 = fma(a1[i], b1[i], s1);
  }
  red[0][threadIdx.x] = s0;
  red[1][threadIdx.x] = s1;
  __syncthreads();
  for (int w = SV_T / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = red[0][0];
    part[2 * blockIdx.x + 1] = red[1][0];
  }
}

// BiCGStab's scalar updates from the dot results; sc holds
// [0] rho, [1] alpha, [2] omega, [3] beta, [4] scratch, [5] ||r||^2 (and the two sums of a k_dot2)
enum { S_RHO = 0, S_ALPHA, S_OMEGA, S_BETA, S_D0, S_D1, S_RR, S_BB, S_N };

__device__ void sum_parts(const double* __restrict__ part, double* out0, double* out1) {
  __shared__ double red[2][SV_T];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < SV_BLOCKS; i += SV_T) {
    a += part[2 * i];
    b += part[2 * i + 1];
  }
  red[0][threadIdx.x] = a;
  red[1][threadIdx.x] = b;
  __syncthreads();
  for (int w = SV_T / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *out0 = red[0][0];
    *out1 = red[1][0];
  }
}

// MODE 0: sc[D0], sc[D1] <- the two sums.  MODE 1 (after (rh, r)): beta = (rho_new / rho) (alpha / omega),
// rho = rho_new.  MODE 2 (after (rh, v)): alpha = rho / (rh, v).  MODE 3 (after (t, s), (t, t)):
// omega = (t, s) / (t, t).  MODE 4: ||r||^2 -> sc[RR].
template <int MODE>
__global__ void k_scalars(const double* __restrict__ part, double* __restrict__ sc) {
  __shared__ double d0, d1;
  sum_parts(part, &d0, &d1);
  __syncthreads();
  if (threadIdx.x != 0) return;
  if (MODE == 0) {
    sc[S_D0] = d0;
    sc[S_D1] = d1;
  } else if (MODE == 1) {
    const double rho_new = d0;
    sc[S_BETA] = (sc[S_RHO] != 0.0 && sc[S_OMEGA] != 0.0) ? (rho_new / sc[S_RHO]) * (sc[S_ALPHA] / sc[S_OMEGA]) : 0.0;
    sc[S_RHO] = rho_new;
  } else if (MODE == 2) {
    sc[S_ALPHA] = d0 != 0.0 ? sc[S_RHO] / d0 : 0.0;
  } else if (MODE == 3) {
    sc[S_OMEGA] = d1 != 0.0 ? d0 / d1 : 0.0;
  } else {
    sc[S_RR] = d0;
  }
}

// p = r + beta (p - omega v)
__global__ void k_update_p(long long n, const double* __restrict__ r, const double* __restrict__ v,
                           double* __restrict__ p, const double* __restrict__ sc) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  p[i] = r[i] + sc[S_BETA] * (p[i] - sc[S_OMEGA] * v[i]);
}
// x += alpha y; s = r - alpha v
__global__ void k_update_xs(long long n, double* __restrict__ x, const double* __restrict__ y,
                            const double* __restrict__ r, const double* __restrict__ v, double* __restrict__ s,
                            const double* __restrict__ sc) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = sc[S_ALPHA];
  x[i] = fma(a, y[i], x[i]);
  s[i] = fma(-a, v[i], r[i]);
}
// x += omega z; r = s - omega t
__global__ void k_update_xr(long long n, double* __restrict__ x, const double* __restrict__ z,
                            const double* __restrict__ s, const double* __restrict__ t, double* __restrict__ r,
                            const double* __restrict__ sc) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double w = sc[S_OMEGA];
  x[i] = fma(w, z[i], x[i]);
  r[i] = fma(-w, t[i], s[i]);
}
// r = b - r (r holds A x on entry), rh = r, p = v = 0; scalars rho = alpha = omega = 1
__global__ void k_init(long long n, const double* __restrict__ b, double* __restrict__ r, double* __restrict__ rh,
                       double* __restrict__ p, double* __restrict__ v, double* __restrict__ sc) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    sc[S_RHO] = 1.0;
    sc[S_ALPHA] = 1.0;
    sc[S_OMEGA] = 1.0;
    sc[S_BETA] = 0.0;
  }
  if (i >= n) return;
  const double ri = b[i] - r[i];
  r[i] = ri;
  rh[i] = ri;
  p[i] = 0.0;
  v[i] = 0.0;
}

template <typename T>
xk_status spmv(const xk_system& A, const double* x, double* y, cudaStream_t st) {
  k_spmv<T><<<xk_blocks(6LL * A.n_nodes, SV_T), SV_T, 0, st>>>(A, x, y);
  return XK_OK;
}

xk_status spmv_any(const xk_system& A, const double* x, double* y, cudaStream_t st) {
  if (A.precision == XK_FP64) return spmv<double>(A, x, y, st);
  return spmv<float>(A, x, y, st);
}

xk_status dot2(long long n, const double* a0, const double* b0, const double* a1, const double* b1, double* part,
               cudaStream_t st) {
  k_dot2<<<SV_BLOCKS, SV_T, 0, st>>>(n, a0, b0, a1, b1, part);
  return XK_OK;
}

}  // namespace

static bool kc_complete(const xk_system* A) {
  return A->kb_blk_row && A->kb_low_ptr && A->kb_low_blk &&
         (!A->kc_vals || (A->kc_row_ptr && A->kc_col && A->kc_blk_row && A->kc_low_ptr && A->kc_low_blk));
}

extern "C" xk_status xk_system_spmv(const xk_system* A, const double* x, double* y, xk_stream s) {
  if (!A || !x || !y || !A->kb_row_ptr || !A->kb_col || !A->kb_vals || !kc_complete(A))
    return xk_set_error(XK_ERR_ARG, "xk_system_spmv: null argument");
  if (A->n_nodes <= 0) return XK_OK;
  spmv_any(*A, x, y, (cudaStream_t)s);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_system_block_jacobi(const xk_system* A, double* dinv, xk_stream s) {
  if (!A || !dinv || !A->kb_row_ptr || !A->kb_col || !A->kb_vals || !kc_complete(A))
    return xk_set_error(XK_ERR_ARG, "xk_system_block_jacobi: null argument");
  if (A->n_nodes <= 0) return XK_OK;
  if (A->precision == XK_FP64)
    k_block_jacobi<double><<<xk_blocks(A->n_nodes, 64), 64, 0, (cudaStream_t)s>>>(*A, dinv);
  else
    k_block_jacobi<float><<<xk_blocks(A->n_nodes, 64), 64, 0, (cudaStream_t)s>>>(*A, dinv);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

namespace {

// One BiCGStab iteration on stream st (scalars on the device).
void bicgstab_iteration(const xk_system& A, long long n, int nb, const double* dinv, double* x, double* r,
                        const double* rh, double* p, double* v, double* y, double* sv, double* z, double* t,
                        double* part, double* sc, cudaStream_t st) {
  dot2(n, rh, r, nullptr, nullptr, part, st);
  k_scalars<1><<<1, SV_T, 0, st>>>(part, sc);  // beta, rho
  k_update_p<<<nb, SV_T, 0, st>>>(n, r, v, p, sc);
  k_apply_block_jacobi<<<nb, SV_T, 0, st>>>(A.n_nodes, dinv, p, y);
  spmv_any(A, y, v, st);
  dot2(n, rh, v, nullptr, nullptr, part, st);
  k_scalars<2><<<1, SV_T, 0, st>>>(part, sc);  // alpha
  k_update_xs<<<nb, SV_T, 0, st>>>(n, x, y, r, v, sv, sc);
  k_apply_block_jacobi<<<nb, SV_T, 0, st>>>(A.n_nodes, dinv, sv, z);
  spmv_any(A, z, t, st);
  dot2(n, t, sv, t, t, part, st);
  k_scalars<3><<<1, SV_T, 0, st>>>(part, sc);  // omega
  k_update_xr<<<nb, SV_T, 0, st>>>(n, x, z, sv, t, r, sc);
}

// ||r||^2 into sc[S_RR]
void residual_sq(long long n, const double* r, double* part, double* sc, cudaStream_t st) {
  dot2(n, r, r, nullptr, nullptr, part, st);
  k_scalars<4><<<1, SV_T, 0, st>>>(part, sc);
}

// A private stream ordered after the caller's, and the graph of one check interval.  On every
// exit, an error return included, the stream is drained before it is destroyed, so that no
// kernel queued on it can still write x or the work vectors after xk_bicgstab has returned.
struct SolveStream {
  cudaStream_t cs = nullptr;
  cudaEvent_t ev = nullptr;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  ~SolveStream() {
    if (cs) cudaStreamSynchronize(cs);
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    if (ev) cudaEventDestroy(ev);
    if (cs) cudaStreamDestroy(cs);
  }
};

}  // namespace

extern "C" xk_status xk_bicgstab(const xk_system* A, const double* b, double* x, const double* dinv, double* work,
                                 int32_t max_iter, int32_t check_every, double rtol, int32_t* iters, double* rel_res,
                                 xk_stream s) {
  if (!A || !b || !x || !dinv || !work || max_iter < 0 || check_every < 1 || !A->kb_row_ptr || !A->kb_col ||
      !A->kb_vals || !kc_complete(A))
    return xk_set_error(XK_ERR_ARG, "xk_bicgstab: bad arguments");
  cudaStream_t st = (cudaStream_t)s;
  const long long n = 6LL * A->n_nodes;
  if (iters) *iters = 0;
  if (rel_res) *rel_res = 0.0;
  if (n == 0) return XK_OK;
  double* r = work;
  double* rh = r + n;
  double* p = rh + n;
  double* v = p + n;
  double* y = v + n;
  double* sv = y + n;
  double* z = sv + n;
  double* t = z + n;
  double* part = t + n;          // [2 * SV_BLOCKS]
  double* sc = part + 2 * SV_BLOCKS;  // [S_N]
  const int nb = xk_blocks(n, SV_T);
  // ||b||^2 and r = b - A x
  dot2(n, b, b, nullptr, nullptr, part, st);
  k_scalars<0><<<1, SV_T, 0, st>>>(part, sc);
  double bb_rr[2];
  XK_CUDA(cudaMemcpyAsync(bb_rr, sc + S_D0, sizeof(double), cudaMemcpyDeviceToHost, st));
  spmv_any(*A, x, r, st);
  k_init<<<nb, SV_T, 0, st>>>(n, b, r, rh, p, v, sc);
  XK_CHECK_LAUNCH();
  XK_CUDA(cudaStreamSynchronize(st));
  const double bb = bb_rr[0] > 0.0 ? bb_rr[0] : 1.0;
  int it = 0;
  double res = 1.0;
  // every check interval (check_every iterations and the residual norm) is one CUDA graph, captured on
  // a private stream; if capture is not possible the same kernels are launched one by one
  SolveStream ss;
  XK_CUDA(cudaStreamCreateWithFlags(&ss.cs, cudaStreamNonBlocking));
  XK_CUDA(cudaEventCreateWithFlags(&ss.ev, cudaEventDisableTiming));
  XK_CUDA(cudaEventRecord(ss.ev, st));
  XK_CUDA(cudaStreamWaitEvent(ss.cs, ss.ev, 0));
  const int interval = check_every < max_iter ? check_every : (max_iter > 0 ? max_iter : 1);
  auto chunk = [&](int k, cudaStream_t cs) {
    for (int q = 0; q < k; ++q) bicgstab_iteration(*A, n, nb, dinv, x, r, rh, p, v, y, sv, z, t, part, sc, cs);
    residual_sq(n, r, part, sc, cs);
  };
  if (max_iter >= interval &&
      cudaStreamBeginCapture(ss.cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    chunk(interval, ss.cs);
    if (cudaStreamEndCapture(ss.cs, &ss.g) != cudaSuccess ||
        cudaGraphInstantiate(&ss.ge, ss.g, 0) != cudaSuccess) {
      ss.ge = nullptr;
      cudaGetLastError();  // capture not possible here: launch one by one
    }
  } else {
    cudaGetLastError();
  }
  while (it < max_iter) {
    const int k = (max_iter - it) < interval ? (max_iter - it) : interval;
    if (ss.ge && k == interval) XK_CUDA(cudaGraphLaunch(ss.ge, ss.cs));
    else chunk(k, ss.cs);
    XK_CHECK_LAUNCH();
    it += k;
    double rr = 0.0;
    XK_CUDA(cudaMemcpyAsync(&rr, sc + S_RR, sizeof(double), cudaMemcpyDeviceToHost, ss.cs));
    XK_CUDA(cudaStreamSynchronize(ss.cs));
    res = sqrt(rr / bb);
    if (!(res > rtol)) break;  // converged (or a NaN, reported through rel_res)
  }
  XK_CUDA(cudaEventRecord(ss.ev, ss.cs));
  XK_CUDA(cudaStreamWaitEvent(st, ss.ev, 0));  // the caller's stream sees x
  if (iters) *iters = it;
  if (rel_res) *rel_res = res;
  return XK_OK;
}

// ---------------------------------------------------------------------------
// The system as dense blocks of a block-tridiagonal matrix, for a direct solve
// on the device.  Nodes are renumbered by pos[] (an ordering along the strand
// axis) and grouped bn to a block; a row of DOFs of node v, DOF d sits in
// block row I = pos[v] / bn at local row 6 (pos[v] % bn) + d.  One thread per
// DOF row writes every entry of its row (K_beam's blocks, then K_c's added on
// the translational part, the mass term on the diagonal), so no entry has two
// writers.  Dirichlet rows and columns become the identity.  A coupling more
// than one block row away cannot be stored: it sets *overflow.
namespace {

template <typename T>
__global__ void k_blocktri(xk_system A, const int32_t* __restrict__ pos, int bn, int nb,
                           const double* __restrict__ mass, double mass_coef, double* __restrict__ D,
                           double* __restrict__ Lo, double* __restrict__ Up, int32_t* __restrict__ overflow) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= 6LL * A.n_nodes) return;
  const int v = (int)(g / 6), d = (int)(g % 6);
  const long long b = 6LL * bn;
  const int pv = pos[v];
  const int I = pv / bn;
  const long long r = 6LL * (pv % bn) + d;
  const long long row_off = (long long)I * b * b + r * b;
  auto at = [&](int w, int j) -> double* {
    const int pw = pos[w];
    const int J = pw / bn;
    const long long c = 6LL * (pw % bn) + j;
    if (J == I) return D + row_off + c;
    if (J == I - 1) return Lo + row_off + c;
    if (J == I + 1) return Up + row_off + c;
    return nullptr;
  };
  if (A.fixed && A.fixed[g]) {  // Dirichlet row: identity (the rest of the row stays zero)
    D[row_off + 6LL * (pv % bn) + d] = 1.0;
    return;
  }
  bool lost = false;
  const T* kb = (const T*)A.kb_vals;
  for (int q = A.kb_low_ptr[v]; q < A.kb_low_ptr[v + 1]; ++q) {  // stored (u, v), u < v, transposed
    const int bk = A.kb_low_blk[q];
    const int u = A.kb_blk_row[bk];
    const T* blk = kb + 36LL * bk + d;
    for (int j = 0; j < 6; ++j) {
      if (A.fixed && A.fixed[6LL * u + j]) continue;
      double* p = at(u, j);
      if (p) *p += (double)blk[6 * j];
      else lost = true;
    }
  }
  for (int bk = A.kb_row_ptr[v]; bk < A.kb_row_ptr[v + 1]; ++bk) {
    const int w = A.kb_col[bk];
    const T* blk = kb + 36LL * bk + 6 * d;
    for (int j = 0; j < 6; ++j) {
      if (A.fixed && A.fixed[6LL * w + j]) continue;
      double* p = at(w, j);
      if (p) *p += (double)blk[j];
      else lost = true;
    }
  }
  if (d < 3 && A.kc_vals) {
    const T* kc = (const T*)A.kc_vals;
    for (int q = A.kc_low_ptr[v]; q < A.kc_low_ptr[v + 1]; ++q) {  // stored (u, v), u < v, also (v, u)
      const int bk = A.kc_low_blk[q];
      const int u = A.kc_blk_row[bk];
      const T* blk = kc + 9LL * bk + 3 * d;
      for (int j = 0; j < 3; ++j) {
        if (A.fixed && A.fixed[6LL * u + j]) continue;
        double* p = at(u, j);
        if (p) *p += (double)blk[j];
        else lost = true;
      }
    }
    for (int bk = A.kc_row_ptr[v]; bk < A.kc_row_ptr[v + 1]; ++bk) {
      const int w = A.kc_col[bk];
      const T* blk = kc + 9LL * bk + 3 * d;
      for (int j = 0; j < 3; ++j) {
        if (A.fixed && A.fixed[6LL * w + j]) continue;
        double* p = at(w, j);
        if (p) *p += (double)blk[j];
        else lost = true;
      }
    }
  }
  if (mass) D[row_off + 6LL * (pv % bn) + d] += mass_coef * mass[g];
  if (lost) atomicExch(overflow, 1);
}

}  // namespace

extern "C" xk_status xk_system_blocktri(const xk_system* A, const int32_t* pos, int32_t bn, int32_t nb,
                                        const double* mass, double mass_coef, double* D, double* Lo, double* Up,
                                        int32_t* overflow, xk_stream s) {
  if (!A || !pos || bn < 1 || nb < 1 || !D || !Lo || !Up || !overflow || !A->kb_row_ptr || !A->kb_col ||
      !A->kb_vals || !kc_complete(A) || (long long)bn * nb < A->n_nodes)
    return xk_set_error(XK_ERR_ARG, "xk_system_blocktri: bad arguments");
  cudaStream_t st = (cudaStream_t)s;
  const long long b = 6LL * bn;
  const size_t bytes = (size_t)nb * b * b * sizeof(double);
  XK_CUDA(cudaMemsetAsync(D, 0, bytes, st));
  XK_CUDA(cudaMemsetAsync(Lo, 0, bytes, st));
  XK_CUDA(cudaMemsetAsync(Up, 0, bytes, st));
  XK_CUDA(cudaMemsetAsync(overflow, 0, sizeof(int32_t), st));
  if (A->n_nodes == 0) return XK_OK;
  const int nbk = xk_blocks(6LL * A->n_nodes, SV_T);
  if (A->precision == XK_FP64)
    k_blocktri<double><<<nbk, SV_T, 0, st>>>(*A, pos, bn, nb, mass, mass_coef, D, Lo, Up, overflow);
  else
    k_blocktri<float><<<nbk, SV_T, 0, st>>>(*A, pos, bn, nb, mass, mass_coef, D, Lo, Up, overflow);
  XK_CHECK_LAUNCH();
  return XK_OK;
}
