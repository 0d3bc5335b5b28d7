// Deterministic, atomic-free reduction of pair contributions into nodal forces
// and the block pattern / values of the contact tangent.
//
// The reference scatters per-pair 12-vectors and 12x12 COO blocks and lets
// np.add.at / scipy sum duplicates (contact_force/strategy.py:161-167,249-253;
// friction/_assembly.py:85-105,119-157,184-257).  Here every pair is reduced
// to v (3) and B (3x3) by the pair kernel, and each node (for forces) or each
// 3x3 node block (for the tangent) sums the pairs incident to it in a fixed
// order: contribution c_k v to node k, and c_k c_l B to block (k, l).
#include "xk_common.cuh"

xk_status xk_sumsq_into(const double* x, long long n, double* out, cudaStream_t s);

namespace {

constexpr int MAX_COLS = 256;  // distinct column nodes per pattern row

XK_D void pair_nodes4(const xk_mesh& m, const xk_pairs& p, int i, int* nd) {
  const int ea = p.ea[i], eb = p.eb[i];
  nd[0] = m.conn[2 * ea];
  nd[1] = m.conn[2 * ea + 1];
  nd[2] = m.conn[2 * eb];
  nd[3] = m.conn[2 * eb + 1];
}

XK_D double shape_c(const xk_pairs& p, int i, int k) {
  const double s = p.s[i], t = p.t[i];
  switch (k) {
    case 0: return 1.0 - s;
    case 1: return s;
    case 2: return -(1.0 - t);
    default: return -t;
  }
}

__global__ void k_member_count(xk_mesh m, xk_pairs p, int32_t* __restrict__ cnt, int32_t* __restrict__ nmem) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool mem = false;
  if (i < p.n) {
    mem = (p.status[i] != 0) || (p.p_n[i] > 0.0);
    if (mem) {
      int nd[4];
      pair_nodes4(m, p, i, nd);
      for (int k = 0; k < 4; ++k) atomicAdd(&cnt[nd[k]], 1);
    }
  }
  unsigned b = __ballot_sync(0xffffffffu, mem);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(nmem, __popc(b));
}

__global__ void k_inc_fill(xk_mesh m, xk_pairs p, const int32_t* __restrict__ ptr, int32_t* __restrict__ fill,
                           int32_t* __restrict__ inc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  if (!((p.status[i] != 0) || (p.p_n[i] > 0.0))) return;
  int nd[4];
  pair_nodes4(m, p, i, nd);
  for (int k = 0; k < 4; ++k) {
    int slot = ptr[nd[k]] + atomicAdd(&fill[nd[k]], 1);
    inc[slot] = (i << 2) | k;
  }
}

// Sort every node's incidence list (insertion sort; lists are short) so that
// all later sums run in pair order, independent of the atomic fill order.
__global__ void k_inc_sort(const int32_t* __restrict__ ptr, int n_nodes, int32_t* __restrict__ inc) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_nodes) return;
  int a = ptr[v], b = ptr[v + 1];
  for (int x = a + 1; x < b; ++x) {
    int key = inc[x], y = x - 1;
    while (y >= a && inc[y] > key) { inc[y + 1] = inc[y]; --y; }
    inc[y + 1] = key;
  }
}

// MODE 0: count the distinct column nodes of each row; MODE 1: write them sorted.
template <int MODE>
__global__ void k_row_cols(xk_mesh m, xk_pairs p, const int32_t* __restrict__ ptr, const int32_t* __restrict__ inc,
                           int n_nodes, int32_t* __restrict__ rcnt, const int32_t* __restrict__ rptr,
                           int32_t* __restrict__ col, int32_t* __restrict__ brow, int32_t* __restrict__ err) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_nodes) return;
  int buf[MAX_COLS];
  int n = 0;
  for (int x = ptr[v]; x < ptr[v + 1]; ++x) {
    int nd[4];
    pair_nodes4(m, p, inc[x] >> 2, nd);
    for (int k = 0; k < 4; ++k) {
      int c = nd[k];
      int y = n - 1;
      while (y >= 0 && buf[y] > c) --y;
      if (y >= 0 && buf[y] == c) continue;
      if (n >= MAX_COLS) { atomicOr(err, 1); continue; }
      for (int z = n - 1; z > y; --z) buf[z + 1] = buf[z];
      buf[y + 1] = c;
      ++n;
    }
  }
  if (MODE == 0) {
    rcnt[v] = n;
  } else {
    int o = rptr[v];
    for (int k = 0; k < n; ++k) {
      col[o + k] = buf[k];
      brow[o + k] = v;
    }
  }
}

template <typename T>
__global__ void k_gather_force(xk_mesh m, xk_pairs p, const int32_t* __restrict__ ptr, const int32_t* __restrict__ inc,
                               const T* __restrict__ pv, int vcol, int vcol2, long long os, const double* __restrict__ base,
                               double scale, const double* __restrict__ f_ext, const uint8_t* __restrict__ fixed,
                               double* __restrict__ out) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.n_nodes) return;
  double acc[3] = {0.0, 0.0, 0.0};
  if (ptr)
    for (int x = ptr[v]; x < ptr[v + 1]; ++x) {
      const int code = inc[x], i = code >> 2, k = code & 3;
      const double c = shape_c(p, i, k);
      for (int d = 0; d < 3; ++d) {
        double w = (double)pv[(vcol + d) * os + i];
        if (vcol2 >= 0) w += (double)pv[(vcol2 + d) * os + i];
        acc[d] += c * w;
      }
    }
  for (int d = 0; d < 6; ++d) {
    const long long dof = 6LL * v + d;
    double r = base ? base[dof] : 0.0;
    if (d < 3) r += scale * acc[d];
    if (f_ext) r -= f_ext[dof];
    if (fixed && fixed[dof]) r = 0.0;
    out[dof] = r;
  }
}

template <typename T>
__global__ void k_gather_tangent(xk_mesh m, xk_pairs p, const int32_t* __restrict__ ptr, const int32_t* __restrict__ inc,
                                 const int32_t* __restrict__ col, const int32_t* __restrict__ brow, long long nnzb,
                                 const T* __restrict__ pB, int bcol, long long os, T* __restrict__ K) {
  long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nnzb) return;
  const int row = brow[b], cn = col[b];
  T acc[9];
  for (int q = 0; q < 9; ++q) acc[q] = T(0);
  for (int x = ptr[row]; x < ptr[row + 1]; ++x) {
    const int code = inc[x], i = code >> 2, k = code & 3;
    int nd[4];
    pair_nodes4(m, p, i, nd);
    const double ck = shape_c(p, i, k);
    for (int l = 0; l < 4; ++l) {
      if (nd[l] != cn) continue;
      const T w = (T)(ck * shape_c(p, i, l));
      for (int q = 0; q < 9; ++q) acc[q] += w * pB[(bcol + q) * os + i];
    }
  }
  for (int q = 0; q < 9; ++q) K[9 * b + q] = acc[q];
}

}  // namespace

extern "C" xk_status xk_contact_pattern_build(const xk_mesh* m, const xk_pairs* p, xk_contact_pattern* pat,
                                              xk_stream s) {
  if (!m || !p || !pat) return xk_set_error(XK_ERR_ARG, "xk_contact_pattern_build: null argument");
  if (!pat->inc_ptr || !pat->row_ptr) return xk_set_error(XK_ERR_ARG, "xk_contact_pattern_build: row arrays missing");
  cudaStream_t st = (cudaStream_t)s;
  const int nn = m->n_nodes;
  pat->n_nodes = nn;
  int32_t *cnt = nullptr, *fill = nullptr, *scal = nullptr;
  int64_t* tot = nullptr;
  XK_CUDA(cudaMallocAsync((void**)&cnt, sizeof(int32_t) * (nn + 1), st));
  XK_CUDA(cudaMallocAsync((void**)&fill, sizeof(int32_t) * (nn + 1), st));
  XK_CUDA(cudaMallocAsync((void**)&scal, sizeof(int32_t) * 2, st));
  XK_CUDA(cudaMallocAsync((void**)&tot, sizeof(int64_t) * 2, st));
  xk_status r = XK_OK;
  int32_t hs[2] = {0, 0};
  int64_t ht[2] = {0, 0};
  auto fail = [&](cudaError_t e) { r = xk_set_cuda_error(e, __FILE__, __LINE__); };
  do {
    cudaError_t e;
    if ((e = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (nn + 1), st)) != cudaSuccess) { fail(e); break; }
    if ((e = cudaMemsetAsync(scal, 0, sizeof(int32_t) * 2, st)) != cudaSuccess) { fail(e); break; }
    if (p->n > 0) k_member_count<<<xk_blocks(p->n, 256), 256, 0, st>>>(*m, *p, cnt, scal);
    if ((e = cudaGetLastError()) != cudaSuccess) { fail(e); break; }
    if ((r = xk_exclusive_scan_i32(cnt, pat->inc_ptr, nn + 1, tot, st)) != XK_OK) break;
    if ((e = cudaMemcpyAsync(hs, scal, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, st)) != cudaSuccess) { fail(e); break; }
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) { fail(e); break; }
    pat->n_members = hs[0];
    if ((long long)hs[0] > pat->cap_members) {
      r = xk_set_error(XK_ERR_CAPACITY, "xk_contact_pattern_build: member capacity too small");
      break;
    }
    if ((e = cudaMemsetAsync(fill, 0, sizeof(int32_t) * (nn + 1), st)) != cudaSuccess) { fail(e); break; }
    if (p->n > 0) k_inc_fill<<<xk_blocks(p->n, 256), 256, 0, st>>>(*m, *p, pat->inc_ptr, fill, pat->inc);
    k_inc_sort<<<xk_blocks(nn, 128), 128, 0, st>>>(pat->inc_ptr, nn, pat->inc);
    k_row_cols<0><<<xk_blocks(nn, 64), 64, 0, st>>>(*m, *p, pat->inc_ptr, pat->inc, nn, cnt, nullptr, nullptr,
                                                     nullptr, scal + 1);
    if ((e = cudaGetLastError()) != cudaSuccess) { fail(e); break; }
    if ((e = cudaMemsetAsync(cnt + nn, 0, sizeof(int32_t), st)) != cudaSuccess) { fail(e); break; }
    if ((r = xk_exclusive_scan_i32(cnt, pat->row_ptr, nn + 1, tot + 1, st)) != XK_OK) break;
    if ((e = cudaMemcpyAsync(ht, tot, sizeof(int64_t) * 2, cudaMemcpyDeviceToHost, st)) != cudaSuccess) { fail(e); break; }
    if ((e = cudaMemcpyAsync(hs, scal, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, st)) != cudaSuccess) { fail(e); break; }
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) { fail(e); break; }
    if (hs[1]) {
      r = xk_set_error(XK_ERR_OVERFLOW, "xk_contact_pattern_build: a node touches more than 256 distinct contact column nodes");
      break;
    }
    pat->nnzb = ht[1];
    if (ht[1] > pat->cap_blocks) {
      r = xk_set_error(XK_ERR_CAPACITY, "xk_contact_pattern_build: block capacity too small");
      break;
    }
    k_row_cols<1><<<xk_blocks(nn, 64), 64, 0, st>>>(*m, *p, pat->inc_ptr, pat->inc, nn, nullptr, pat->row_ptr,
                                                     pat->col, pat->blk_row, scal + 1);
    if ((e = cudaGetLastError()) != cudaSuccess) { fail(e); break; }
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) { fail(e); break; }
  } while (0);
  cudaFreeAsync(cnt, st);
  cudaFreeAsync(fill, st);
  cudaFreeAsync(scal, st);
  cudaFreeAsync(tot, st);
  return r;
}

extern "C" xk_status xk_contact_gather_force(const xk_mesh* m, const xk_pairs* p, const xk_contact_pattern* pat,
                                             const void* pv, int precision, int out_mode, int which,
                                             int64_t out_stride, const double* base, double scale,
                                             const double* f_ext, const uint8_t* fixed, double* out, double* norm2,
                                             xk_stream s) {
  if (!m || !p || !out) return xk_set_error(XK_ERR_ARG, "xk_contact_gather_force: null argument");
  int vcol = 0, vcol2 = -1;
  if (out_mode == XK_OUT_SPLIT) {
    if (which == XK_WHICH_NORMAL) vcol = 0;
    else if (which == XK_WHICH_FRICTION) vcol = 3;
    else { vcol = 0; vcol2 = 3; }
  } else if (which != XK_WHICH_COMBINED) {
    return xk_set_error(XK_ERR_ARG, "xk_contact_gather_force: combined output holds only the combined force");
  }
  const bool use_pairs = pat && pat->n_members > 0 && pv;
  const int32_t* ptr = use_pairs ? pat->inc_ptr : nullptr;
  const int32_t* inc = use_pairs ? pat->inc : nullptr;
  cudaStream_t st = (cudaStream_t)s;
  if (m->n_nodes > 0) {
    if (precision == XK_FP64)
      k_gather_force<double><<<xk_blocks(m->n_nodes, 128), 128, 0, st>>>(*m, *p, ptr, inc, (const double*)pv, vcol,
                                                                          vcol2, out_stride, base, scale, f_ext, fixed,
                                                                          out);
    else if (precision == XK_MIXED)
      k_gather_force<float><<<xk_blocks(m->n_nodes, 128), 128, 0, st>>>(*m, *p, ptr, inc, (const float*)pv, vcol,
                                                                         vcol2, out_stride, base, scale, f_ext, fixed,
                                                                         out);
    else
      return xk_set_error(XK_ERR_ARG, "xk_contact_gather_force: precision");
    XK_CHECK_LAUNCH();
  }
  if (norm2) return xk_sumsq_into(out, 6LL * m->n_nodes, norm2, st);
  return XK_OK;
}

extern "C" xk_status xk_contact_gather_tangent(const xk_mesh* m, const xk_pairs* p, const xk_contact_pattern* pat,
                                               const void* pB, int precision, int out_mode, int which,
                                               int64_t out_stride, void* Kc_vals, xk_stream s) {
  if (!m || !p || !pat || !pB || !Kc_vals) return xk_set_error(XK_ERR_ARG, "xk_contact_gather_tangent: null argument");
  int bcol = 0;
  if (out_mode == XK_OUT_SPLIT) {
    if (which == XK_WHICH_NORMAL) bcol = 0;
    else if (which == XK_WHICH_FRICTION) bcol = 9;
    else return xk_set_error(XK_ERR_ARG, "xk_contact_gather_tangent: split output needs which = normal or friction");
  } else if (which != XK_WHICH_COMBINED) {
    return xk_set_error(XK_ERR_ARG, "xk_contact_gather_tangent: combined output holds only the combined tangent");
  }
  if (pat->nnzb == 0) return XK_OK;
  cudaStream_t st = (cudaStream_t)s;
  const int nb = xk_blocks(pat->nnzb, 128);
  if (precision == XK_FP64)
    k_gather_tangent<double><<<nb, 128, 0, st>>>(*m, *p, pat->inc_ptr, pat->inc, pat->col, pat->blk_row, pat->nnzb,
                                                 (const double*)pB, bcol, out_stride, (double*)Kc_vals);
  else if (precision == XK_MIXED)
    k_gather_tangent<float><<<nb, 128, 0, st>>>(*m, *p, pat->inc_ptr, pat->inc, pat->col, pat->blk_row, pat->nnzb,
                                                (const float*)pB, bcol, out_stride, (float*)Kc_vals);
  else
    return xk_set_error(XK_ERR_ARG, "xk_contact_gather_tangent: precision");
  XK_CHECK_LAUNCH();
  return XK_OK;
}
