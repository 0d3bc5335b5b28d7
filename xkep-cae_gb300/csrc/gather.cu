// Per-increment contact pattern and the deterministic, atomic-free reduction of
// pair contributions into nodal forces and 3x3 contact-tangent blocks.
//
// The reference scatters per-pair 12-vectors and 12x12 COO blocks and lets
// np.add.at / scipy sum the duplicates (contact_force/strategy.py:161-167,249-253;
// friction/_assembly.py:85-105,119-157,184-257).  Here the pair kernel reduces
// every contributing pair ("member") to a record (s, t, v, B): its force on
// local node k is c_k v and its tangent block (k, l) is c_k c_l B with
// c = [1-s, s, -(1-t), -t].  Each node sums its incident members and each
// K_c block sums its contributor list, both in a fixed order.
//
// Every contribution to block (v, w) is c_k c_l B and the same member gives
// c_l c_k B to block (w, v): the block at (w, v) equals the block at (v, w)
// (the same 3x3 values, not the transpose; K_c itself is not symmetric once
// friction acts).  So the pattern holds the blocks with row <= column only
// ("upper" blocks), each computed once, and a lower index lists, per node w,
// the stored blocks (v, w) with v < w, for readers that need whole rows.
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

template <typename T>
XK_D T shape_c(T s, T t, int k) {
  switch (k) {
    case 0: return T(1) - s;
    case 1: return s;
    case 2: return -(T(1) - t);
    default: return -t;
  }
}

// A pair contributes in the increment when it is not INACTIVE or still carries a normal force; with
// coated wires every pair does, since the reference evaluates the coating force of every pair.
XK_D bool is_member(const xk_pairs& p, int i) {
  return (p.status[i] != 0) || (p.p_n[i] > 0.0) || (p.coat_cc != nullptr);
}

__global__ void k_flags(xk_pairs p, int32_t* __restrict__ flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < p.n) flag[i] = is_member(p, i) ? 1 : 0;
  else if (i == p.n) flag[i] = 0;
}

__global__ void k_split_lists(xk_mesh m, xk_pairs p, const int32_t* __restrict__ mpos, int32_t* __restrict__ members,
                              int32_t* __restrict__ mnodes, int32_t* __restrict__ others) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int k = mpos[i];
  if (is_member(p, i)) {
    members[k] = i;
    int nd[4];
    pair_nodes4(m, p, i, nd);
    for (int q = 0; q < 4; ++q) mnodes[4LL * k + q] = nd[q];
  } else {
    others[i - k] = i;
  }
}

__global__ void k_inc_count(const int32_t* __restrict__ mnodes, int nm, int32_t* __restrict__ cnt) {
  int mi = blockIdx.x * blockDim.x + threadIdx.x;
  if (mi >= nm) return;
  for (int k = 0; k < 4; ++k) atomicAdd(&cnt[mnodes[4LL * mi + k]], 1);
}

__global__ void k_inc_fill(const int32_t* __restrict__ mnodes, int nm, const int32_t* __restrict__ ptr,
                           int32_t* __restrict__ fill, int32_t* __restrict__ inc) {
  int mi = blockIdx.x * blockDim.x + threadIdx.x;
  if (mi >= nm) return;
  for (int k = 0; k < 4; ++k) {
    const int v = mnodes[4LL * mi + k];
    inc[ptr[v] + atomicAdd(&fill[v], 1)] = (mi << 2) | k;
  }
}

// Sort every segment [ptr[v], ptr[v+1]) ascending, so that sums run in a fixed order whatever the
// order of the atomic fill.  A warp per segment: up to 64 entries (the entries of a segment are
// distinct) sit in two registers per lane and each finds its rank by comparing against all others
// broadcast by shuffles, then the warp writes them to their ranks; a longer segment is sorted by
// insertion by one lane.
constexpr int SEG_T = 128;
XK_D void warp_sort_segment(int lo, int hi, int32_t* __restrict__ a, int lane) {
  const int n = hi - lo;
  if (n <= 1) return;
  if (n > 64) {
    if (lane == 0) {
      for (int x = lo + 1; x < hi; ++x) {
        const int key = a[x];
        int y = x - 1;
        while (y >= lo && a[y] > key) { a[y + 1] = a[y]; --y; }
        a[y + 1] = key;
      }
    }
    return;
  }
  const int v0 = lane < n ? a[lo + lane] : 0x7fffffff;
  const int v1 = lane + 32 < n ? a[lo + lane + 32] : 0x7fffffff;
  int r0 = 0, r1 = 0;
  const int n0 = n < 32 ? n : 32;
  for (int k = 0; k < n0; ++k) {
    const int x = __shfl_sync(0xffffffffu, v0, k);
    r0 += x < v0;
    r1 += x < v1;
  }
  for (int k = 0; k < n - 32; ++k) {
    const int x = __shfl_sync(0xffffffffu, v1, k);
    r0 += x < v0;
    r1 += x < v1;
  }
  __syncwarp();
  if (lane < n) a[lo + r0] = v0;
  if (lane + 32 < n) a[lo + r1] = v1;
}

__global__ void __launch_bounds__(SEG_T) k_segment_sort(const int32_t* __restrict__ ptr, long long nseg,
                                                        int32_t* __restrict__ a) {
  const long long v = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (v >= nseg) return;
  warp_sort_segment(ptr[v], ptr[v + 1], a, threadIdx.x & 31);
}

// The same sort for many short segments (the contributor lists of the blocks, a few entries each, where a
// warp per segment spends its time on warps): a thread per segment sorts one of at most SEG_SHORT entries
// by insertion in place and lists a longer one (a diagonal block, one entry per member at the node) for
// k_segment_sort_listed, whose persistent warps take the listed segments in turn.
constexpr int SEG_SHORT = 12;
__global__ void k_segment_sort_short(const int32_t* __restrict__ ptr, long long nseg, int32_t* __restrict__ a,
                                     int32_t* __restrict__ longs, int32_t* __restrict__ n_longs) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nseg) return;
  const int lo = ptr[v], hi = ptr[v + 1];
  if (hi - lo > SEG_SHORT) {
    longs[atomicAdd(n_longs, 1)] = (int)v;
    return;
  }
  for (int x = lo + 1; x < hi; ++x) {
    const int key = a[x];
    int y = x - 1;
    while (y >= lo && a[y] > key) { a[y + 1] = a[y]; --y; }
    a[y + 1] = key;
  }
}

__global__ void __launch_bounds__(SEG_T) k_segment_sort_listed(const int32_t* __restrict__ ptr,
                                                               int32_t* __restrict__ a,
                                                               const int32_t* __restrict__ longs,
                                                               const int32_t* __restrict__ n_longs) {
  const int n = *n_longs;
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (SEG_T / 32);
  for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n; w += nw) {
    const int v = longs[w];
    warp_sort_segment(ptr[v], ptr[v + 1], a, lane);
  }
}

// The distinct column nodes c >= v of row v, in ascending order, from its member incidences (the four nodes
// of every member touching v).  A warp per node: the candidates >= v (4 per incidence, at most RC_CAP) go
// into a per-warp open-addressing hash set in shared memory (twice the candidates' power of two, linear
// probing, atomicCAS among the warp's lanes), which drops the repeats; the distinct values are gathered
// by a ballot scan of the set and ranked: by shuffles when at most 64 (two per lane), else by a bitonic
// sort in shared memory.  MODE 0 counts them (rcnt[v]); MODE 1 writes them at rptr[v] (col, and v in
// brow).  A node with more than RC_CAP candidates takes the serial path of one lane (insertion into a
// sorted local buffer of MAX_COLS distinct columns; err bit 1 if that overflows).
constexpr int RC_WARPS = 4, RC_CAP = 512, RC_TAB = 2 * RC_CAP;
XK_D int row_cols_serial(const int32_t* __restrict__ mnodes, const int32_t* __restrict__ inc, int x0, int x1, int v,
                         int* buf, int32_t* __restrict__ err) {
  int n = 0;
  for (int x = x0; x < x1; ++x) {
    const long long mi = inc[x] >> 2;
    for (int k = 0; k < 4; ++k) {
      const int c = mnodes[4 * mi + k];
      if (c < v) continue;
      int y = n - 1;
      while (y >= 0 && buf[y] > c) --y;
      if (y >= 0 && buf[y] == c) continue;
      if (n >= MAX_COLS) { atomicOr(err, 1); continue; }
      for (int z = n - 1; z > y; --z) buf[z + 1] = buf[z];
      buf[y + 1] = c;
      ++n;
    }
  }
  return n;
}

template <int MODE>
__global__ void __launch_bounds__(32 * RC_WARPS) k_row_cols(const int32_t* __restrict__ mnodes,
                                                            const int32_t* __restrict__ ptr,
                                                            const int32_t* __restrict__ inc, int n_nodes,
                                                            int32_t* __restrict__ rcnt,
                                                            const int32_t* __restrict__ rptr,
                                                            int32_t* __restrict__ col, int32_t* __restrict__ brow,
                                                            int32_t* __restrict__ err) {
  __shared__ int stab[RC_WARPS][RC_TAB];
  __shared__ int slist[RC_WARPS][RC_CAP];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int v = blockIdx.x * RC_WARPS + wid;
  if (v >= n_nodes) return;
  const int x0 = ptr[v], x1 = ptr[v + 1];
  const int nc = 4 * (x1 - x0);
  if (nc > RC_CAP) {
    if (lane == 0) {
      int buf[MAX_COLS];
      const int n = row_cols_serial(mnodes, inc, x0, x1, v, buf, err);
      if (MODE == 0) {
        rcnt[v] = n;
      } else {
        for (int k = 0; k < n; ++k) {
          col[rptr[v] + k] = buf[k];
          brow[rptr[v] + k] = v;
        }
      }
    }
    return;
  }
  constexpr int EMPTY = -1;
  int* t = stab[wid];
  int* l = slist[wid];
  int ts = 64;
  while (ts < 2 * nc) ts <<= 1;  // a power of two, at least twice the candidates
  for (int i = lane; i < ts; i += 32) t[i] = EMPTY;
  __syncwarp();
  for (int i = lane; i < nc; i += 32) {
    const int c = mnodes[4LL * (inc[x0 + (i >> 2)] >> 2) + (i & 3)];
    if (c < v) continue;
    unsigned h = ((unsigned)c * 2654435761u) & (unsigned)(ts - 1);
    while (true) {
      const int o = atomicCAS(&t[h], EMPTY, c);
      if (o == EMPTY || o == c) break;
      h = (h + 1) & (unsigned)(ts - 1);
    }
  }
  __syncwarp();
  int nd = 0;
  const unsigned below = (1u << lane) - 1u;
  for (int i0 = 0; i0 < ts; i0 += 32) {
    const int x = t[i0 + lane];
    const unsigned bal = __ballot_sync(0xffffffffu, x != EMPTY);
    if (x != EMPTY) l[nd + __popc(bal & below)] = x;
    nd += __popc(bal);
  }
  __syncwarp();
  if (MODE == 0) {
    if (lane == 0) rcnt[v] = nd;
    return;
  }
  const int o = rptr[v];
  if (nd <= 64) {  // ranks by shuffle-broadcast comparisons (the values are distinct)
    const int v0 = lane < nd ? l[lane] : 0x7fffffff;
    const int v1 = lane + 32 < nd ? l[lane + 32] : 0x7fffffff;
    int r0 = 0, r1 = 0;
    const int n0 = nd < 32 ? nd : 32;
    for (int k = 0; k < n0; ++k) {
      const int x = __shfl_sync(0xffffffffu, v0, k);
      r0 += x < v0;
      r1 += x < v1;
    }
    for (int k = 0; k < nd - 32; ++k) {
      const int x = __shfl_sync(0xffffffffu, v1, k);
      r0 += x < v0;
      r1 += x < v1;
    }
    if (lane < nd) { col[o + r0] = v0; brow[o + r0] = v; }
    if (lane + 32 < nd) { col[o + r1] = v1; brow[o + r1] = v; }
    return;
  }
  int N = 32;
  while (N < nd) N <<= 1;
  for (int i = nd + lane; i < N; i += 32) l[i] = 0x7fffffff;
  __syncwarp();
  for (int k = 2; k <= N; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < N; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const int p = l[i], q = l[ixj];
          if (((i & k) == 0) == (p > q)) {
            l[i] = q;
            l[ixj] = p;
          }
        }
      }
      __syncwarp();
    }
  for (int i = lane; i < nd; i += 32) {
    col[o + i] = l[i];
    brow[o + i] = v;
  }
}

// Lower index: per node w, the stored blocks (v, w) with v < w in the order of v (MODE 0 counts).
template <int MODE>
__global__ void k_lower_index(long long nb, const int32_t* __restrict__ brow, const int32_t* __restrict__ col,
                              int32_t* __restrict__ cnt, const int32_t* __restrict__ lptr, int32_t* __restrict__ lblk) {
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const int w = col[b];
  if (brow[b] == w) return;
  if (MODE == 0) atomicAdd(&cnt[w], 1);
  else lblk[lptr[w] + atomicAdd(&cnt[w], 1)] = (int)b;
}

XK_D int find_block(const int32_t* __restrict__ rptr, const int32_t* __restrict__ col, int row, int c) {
  int lo = rptr[row], hi = rptr[row + 1];
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (col[mid] < c) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// MODE 0: count contributions per block; MODE 1: fill (member << 4 | k << 2 | l).
template <int MODE>
__global__ void k_contrib(const int32_t* __restrict__ mnodes, int nm, const int32_t* __restrict__ rptr,
                          const int32_t* __restrict__ col, int32_t* __restrict__ cnt,
                          const int32_t* __restrict__ bptr, int32_t* __restrict__ contrib, int32_t* __restrict__ err) {
  int mi = blockIdx.x * blockDim.x + threadIdx.x;
  if (mi >= nm) return;
  int nd[4];
  for (int q = 0; q < 4; ++q) nd[q] = mnodes[4LL * mi + q];
  for (int k = 0; k < 4; ++k)
    for (int l = 0; l < 4; ++l) {
      if (nd[k] > nd[l]) continue;  // a lower block: the same values as its stored mirror
      const int b = find_block(rptr, col, nd[k], nd[l]);
      if (b >= rptr[nd[k] + 1] || col[b] != nd[l]) {  // cannot happen for a consistent pattern
        atomicOr(err, 2);
        continue;
      }
      if (MODE == 0) {
        atomicAdd(&cnt[b], 1);
      } else {
        contrib[bptr[b] + atomicAdd(&cnt[b], 1)] = (mi << 4) | (k << 2) | l;
      }
    }
}

// Mesh node -> (element, local index, other node) lists, and member sides per element.
__global__ void k_node_elem_count(xk_mesh m, int32_t* __restrict__ cnt) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.n_elems) return;
  atomicAdd(&cnt[m.conn[2 * e]], 1);
  atomicAdd(&cnt[m.conn[2 * e + 1]], 1);
}

__global__ void k_node_elem_fill(xk_mesh m, const int32_t* __restrict__ ptr, int32_t* __restrict__ fill,
                                 int2* __restrict__ ne) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.n_elems) return;
  for (int p = 0; p < 2; ++p) {
    const int v = m.conn[2 * e + p];
    ne[ptr[v] + atomicAdd(&fill[v], 1)] = make_int2((e << 1) | p, m.conn[2 * e + 1 - p]);
  }
}

__global__ void k_segment_sort_pairs(const int32_t* __restrict__ ptr, long long nseg, int2* __restrict__ a) {
  long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nseg) return;
  const int lo = ptr[v], hi = ptr[v + 1];
  for (int x = lo + 1; x < hi; ++x) {
    const int2 key = a[x];
    int y = x - 1;
    while (y >= lo && a[y].x > key.x) { a[y + 1] = a[y]; --y; }
    a[y + 1] = key;
  }
}

__global__ void k_elem_inc_count(xk_pairs p, const int32_t* __restrict__ members, int nm, int32_t* __restrict__ cnt) {
  const int mi = blockIdx.x * blockDim.x + threadIdx.x;
  if (mi >= nm) return;
  const int i = members[mi];
  atomicAdd(&cnt[p.ea[i]], 1);
  atomicAdd(&cnt[p.eb[i]], 1);
}

__global__ void k_elem_inc_fill(xk_pairs p, const int32_t* __restrict__ members, int nm,
                                const int32_t* __restrict__ ptr, int32_t* __restrict__ fill,
                                int32_t* __restrict__ inc) {
  const int mi = blockIdx.x * blockDim.x + threadIdx.x;
  if (mi >= nm) return;
  const int i = members[mi];
  const int ea = p.ea[i], eb = p.eb[i];
  inc[ptr[ea] + atomicAdd(&fill[ea], 1)] = mi << 1;
  inc[ptr[eb] + atomicAdd(&fill[eb], 1)] = (mi << 1) | 1;
}

// One member record (16 values for combined records) through vector loads.
template <typename T, int N>
XK_D void load_rec(const T* __restrict__ r, T* out);
template <>
XK_D void load_rec<float, 16>(const float* __restrict__ r, float* out) {
  const float4* p = reinterpret_cast<const float4*>(r);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 v = __ldg(p + i);
    out[4 * i] = v.x; out[4 * i + 1] = v.y; out[4 * i + 2] = v.z; out[4 * i + 3] = v.w;
  }
}
template <>
XK_D void load_rec<double, 16>(const double* __restrict__ r, double* out) {
  const double2* p = reinterpret_cast<const double2*>(r);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const double2 v = __ldg(p + i);
    out[2 * i] = v.x; out[2 * i + 1] = v.y;
  }
}

// Eight lanes per node: lane l of the group takes incidences l, l+8, ...; the
// group's partial sums are combined by a fixed shuffle tree, so the result does
// not depend on timing.  Sums run in the record precision T (the mixed path
// accumulates in float) and are converted once per degree of freedom.
constexpr int GF_LANES = 8;
template <typename T>
__global__ void k_gather_force(int n_nodes, const int32_t* __restrict__ ptr, const int32_t* __restrict__ inc,
                               const T* __restrict__ rec, int rs, int stc, int vcol, int vcol2,
                               const double* __restrict__ base, double scale, const double* __restrict__ f_ext,
                               const uint8_t* __restrict__ fixed, double* __restrict__ out) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int v = gid / GF_LANES, lane = gid % GF_LANES;
  const bool live = v < n_nodes;
  T acc[3] = {T(0), T(0), T(0)};
  if (live && ptr)
    for (int x = ptr[v] + lane; x < ptr[v + 1]; x += GF_LANES) {
      const int code = inc[x], k = code & 3;
      const T* r = rec + (long long)(code >> 2) * rs;
      const T c = shape_c<T>(r[stc], r[stc + 1], k);
      for (int d = 0; d < 3; ++d) {
        T w = r[vcol + d];
        if (vcol2 >= 0) w += r[vcol2 + d];
        acc[d] += c * w;
      }
    }
#pragma unroll
  for (int o = GF_LANES / 2; o > 0; o >>= 1)
#pragma unroll
    for (int d = 0; d < 3; ++d) acc[d] += __shfl_down_sync(0xffffffffu, acc[d], o, GF_LANES);
#pragma unroll
  for (int d = 0; d < 3; ++d) acc[d] = __shfl_sync(0xffffffffu, acc[d], 0, GF_LANES);
  if (live && lane < 6) {
    const int d = lane;
    const long long dof = 6LL * v + d;
    double r = base ? base[dof] : 0.0;
    if (d < 3) r += scale * (double)(d == 0 ? acc[0] : (d == 1 ? acc[1] : acc[2]));
    if (f_ext) r -= f_ext[dof];
    if (fixed && fixed[dof]) r = 0.0;
    out[dof] = r;
  }
}

// Column of s (then t) in a record of RS values: combined records put B first.
template <int RS>
__host__ __device__ constexpr int rec_st() { return RS == XK_REC_STRIDE_COMBINED ? XK_REC_S : 0; }

template <typename T, int RS, int BCOL>
XK_D void add_contrib(const T* __restrict__ rec, int code, T* acc) {
  constexpr int ST = rec_st<RS>();
  const int k = (code >> 2) & 3, l = code & 3;
  T r[RS];
  if (RS == 16) {
    load_rec<T, 16>(rec + (long long)(code >> 4) * RS, r);
  } else {
#pragma unroll
    for (int q = 0; q < RS; ++q) r[q] = rec[(long long)(code >> 4) * RS + q];
  }
  const T w = shape_c<T>(r[ST], r[ST + 1], k) * shape_c<T>(r[ST], r[ST + 1], l);
#pragma unroll
  for (int q = 0; q < 9; ++q) acc[q] += w * r[BCOL + q];
}

// Inline term lists of the blocks (variant "sides").  k_side_codes writes the
// same-side terms of every block (diagonal: S^pp of each element of the row
// node; neighbour on an element: S^01) and the count; k_cross_codes appends
// the cross codes of every member; k_sort_codes sorts each block's four slots.
constexpr int SIDE_FLAG = (int)0x80000000;
// An element's three sums S^00, S^01, S^11, each as 16 values: the 9 of the
// sum, then 1, 1 in the places of a record's s, t and padding, so that a term
// loads the same values from an element sum as from a combined record (both
// 64-byte aligned) and the weight c_1 c_1 = s s of an element-sum term is 1.
constexpr int SUM_STRIDE = 16;
constexpr int ELEM_SUMS = 3 * SUM_STRIDE;

__global__ void k_side_codes(long long nb, const int32_t* __restrict__ brow, const int32_t* __restrict__ col,
                             const int32_t* __restrict__ neptr, const int2* __restrict__ ne,
                             int32_t* __restrict__ codes, int32_t* __restrict__ cnt, int32_t* __restrict__ err) {
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const int i = brow[b], j = col[b];
  int n = 0;
  for (int y = neptr[i]; y < neptr[i + 1]; ++y) {
    const int2 en = ne[y];
    const int base = ELEM_SUMS * (en.x >> 1);
    if (j == i) {
      if (n < 4) codes[4 * b + n] = SIDE_FLAG | (base + ((en.x & 1) ? 2 * SUM_STRIDE : 0));
      ++n;
    }
    if (j == en.y) {
      if (n < 4) codes[4 * b + n] = SIDE_FLAG | (base + SUM_STRIDE);
      ++n;
    }
  }
  if (n > 4) atomicOr(err, 1);
  cnt[b] = n;
}

__global__ void k_cross_codes(const int32_t* __restrict__ mnodes, int nm, const int32_t* __restrict__ rptr,
                              const int32_t* __restrict__ col, int32_t* __restrict__ cnt,
                              int32_t* __restrict__ codes, int32_t* __restrict__ err) {
  const int mi = blockIdx.x * blockDim.x + threadIdx.x;
  if (mi >= nm) return;
  int nd[4];
  for (int q = 0; q < 4; ++q) nd[q] = mnodes[4LL * mi + q];
  for (int k = 0; k < 4; ++k)
    for (int l = 0; l < 4; ++l) {
      if ((k >> 1) == (l >> 1) || nd[k] > nd[l]) continue;
      const int b = find_block(rptr, col, nd[k], nd[l]);
      if (b >= rptr[nd[k] + 1] || col[b] != nd[l]) {
        atomicOr(err, 2);
        continue;
      }
      const int slot = atomicAdd(&cnt[b], 1);
      if (slot < 4) codes[4LL * b + slot] = (mi << 4) | (k << 2) | l;
      else atomicOr(err, 1);
    }
}

__global__ void k_sort_codes(long long nb, int4* __restrict__ codes) {
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  int4 c = codes[b];
  int v[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
  for (int x = 1; x < 4; ++x)
#pragma unroll
    for (int y = x; y > 0; --y)
      if (v[y - 1] > v[y]) { const int t = v[y]; v[y] = v[y - 1]; v[y - 1] = t; }
  codes[b] = make_int4(v[0], v[1], v[2], v[3]);
}

// Variant "sides", step 1: S_e^00, S_e^01, S_e^11 (9 values each) of every
// element from its members, one thread per (element, B component); the weights
// are the products c_p c_q of the member's side: (1-s)^2, (1-s)s, s^2 on side A
// and the same in t on side B (the signs of c_2, c_3 cancel).
//
// With combined records the same pass also forms the element's force sums
// F_e^0 = sum c_p v and F_e^1 = sum c_q v over its members (p, q the element's
// first and second local node on the member's side: c = 1-s, s on side A and
// -(1-t), -t on side B), 8 values per element after the 36 * ne tangent sums;
// a node's contact force is then the sum of F over its incident elements
// (k_gather_force_elem).
constexpr int ELEM_FORCE = 8;

template <typename T, int RS, int BCOL>
__global__ void k_elem_sums(int ne, const int32_t* __restrict__ eptr, const int32_t* __restrict__ einc,
                            const T* __restrict__ rec, T* __restrict__ S) {
  constexpr int ST = rec_st<RS>();
  constexpr bool FORCE = RS == XK_REC_STRIDE_COMBINED;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 9LL * ne) return;
  const int e = (int)(t / 9), q = (int)(t % 9);
  T s00 = T(0), s01 = T(0), s11 = T(0), f0 = T(0), f1 = T(0);
  const int x1 = eptr[e + 1];
#pragma unroll 4
  for (int x = eptr[e]; x < x1; ++x) {
    const int code = einc[x];
    const T* r = rec + (long long)(code >> 1) * RS;
    const T a = r[ST + (code & 1)];
    const T b = r[BCOL + q];
    const T om = T(1) - a;
    s00 += (om * om) * b;
    s01 += (om * a) * b;
    s11 += (a * a) * b;
    if (FORCE && q < 3) {
      const T v = (code & 1) ? -r[XK_REC_V + q] : r[XK_REC_V + q];
      f0 += om * v;
      f1 += a * v;
    }
  }
  T* o = S + (long long)ELEM_SUMS * e;
  o[q] = s00;
  o[SUM_STRIDE + q] = s01;
  o[2 * SUM_STRIDE + q] = s11;
  if (q < 3) {  // padding of sum q: (s, t) = (1, 1)
    o[q * SUM_STRIDE + 9] = T(1);
    o[q * SUM_STRIDE + 10] = T(1);
    if (FORCE) {
      T* f = S + (long long)ELEM_SUMS * ne + (long long)ELEM_FORCE * e;
      f[q] = f0;
      f[3 + q] = f1;
      if (q < 2) f[6 + q] = T(0);
    }
  }
}

// The same sums for combined records, four lanes per element: lane q sums the incidences
// q, q + 4, q + 8, ... of the element (each one record read as two 256-bit loads for float),
// and the four partial sums are combined by a fixed shuffle tree ((q + q^2) + (q^1 + q^3)), so the
// result does not depend on timing.  It differs from k_elem_sums' single running sum by
// rounding only.
template <typename T>
XK_D void load16(const T* __restrict__ p, T* v);
template <>
XK_D void load16<float>(const float* __restrict__ p, float* v) {  // p 32-byte aligned
  ldg8(p, v);
  ldg8(p + 8, v + 8);
}
template <>
XK_D void load16<double>(const double* __restrict__ p, double* v) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const double2 x = __ldg(q + i);
    v[2 * i] = x.x; v[2 * i + 1] = x.y;
  }
}

template <typename T>
XK_D void store4(T* p, T a, T b, T c, T d);
template <>
XK_D void store4<float>(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
template <>
XK_D void store4<double>(double* p, double a, double b, double c, double d) {
  reinterpret_cast<double2*>(p)[0] = make_double2(a, b);
  reinterpret_cast<double2*>(p)[1] = make_double2(c, d);
}

template <typename T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 7 : 4) k_elem_sums_rec(int ne, const int32_t* __restrict__ eptr,
                                                       const int32_t* __restrict__ einc, const T* __restrict__ rec,
                                                       T* __restrict__ S) {
  static_assert(XK_REC_B == 0 && XK_REC_S == 9 && XK_REC_V == 11, "combined record layout");
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int e = (int)(gid >> 2), q = (int)(gid & 3);
  const bool live = e < ne;  // a quad is all live or all dead (4 | 128)
  T s00[9], s01[9], s11[9], f0[3], f1[3];
#pragma unroll
  for (int c = 0; c < 9; ++c) { s00[c] = T(0); s01[c] = T(0); s11[c] = T(0); }
#pragma unroll
  for (int c = 0; c < 3; ++c) { f0[c] = T(0); f1[c] = T(0); }
  const int x0 = live ? eptr[e] : 0, x1 = live ? eptr[e + 1] : 0;
  // two incidences per round (x and x + 4), both records loaded before either is summed; the
  // sums still take the lane's incidences in order
  for (int x = x0 + q; x < x1; x += 8) {
    const bool two = x + 4 < x1;
    const int code0 = einc[x];
    const int code1 = two ? einc[x + 4] : code0;
    T r[2][16];
    load16<T>(rec + (long long)(code0 >> 1) * XK_REC_STRIDE_COMBINED, r[0]);
    if (two) load16<T>(rec + (long long)(code1 >> 1) * XK_REC_STRIDE_COMBINED, r[1]);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      if (j == 1 && !two) break;
      const int code = j == 0 ? code0 : code1;
      const T a = (code & 1) ? r[j][XK_REC_S + 1] : r[j][XK_REC_S];
      const T om = T(1) - a;
#pragma unroll
      for (int c = 0; c < 9; ++c) {
        s00[c] += (om * om) * r[j][c];
        s01[c] += (om * a) * r[j][c];
        s11[c] += (a * a) * r[j][c];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const T v = (code & 1) ? -r[j][XK_REC_V + c] : r[j][XK_REC_V + c];
        f0[c] += om * v;
        f1[c] += a * v;
      }
    }
  }
  // Reduce-scatter over the quad: the 33 sums (S^00, S^01, S^11, F^0, F^1, padded to 36) split in
  // halves between lanes q and q ^ 2, then in quarters between q and q ^ 1, so that lane q ends with
  // the nine values it stores (lane 0 S^00, 1 S^01, 2 S^11, 3 F^0 F^1) as (l_q + l_q^2) +
  // (l_q^1 + l_q^3): a fixed tree of 27 shuffles per lane.
  T v[36];
#pragma unroll
  for (int c = 0; c < 9; ++c) { v[c] = s00[c]; v[9 + c] = s01[c]; v[18 + c] = s11[c]; }
#pragma unroll
  for (int c = 0; c < 3; ++c) { v[27 + c] = f0[c]; v[30 + c] = f1[c]; v[33 + c] = T(0); }
  const bool hi = (q >> 1) & 1, odd = q & 1;
#pragma unroll
  for (int c = 0; c < 18; ++c) {  // lane q keeps half hi, receives it from q ^ 2
    const T y = __shfl_xor_sync(0xffffffffu, hi ? v[c] : v[18 + c], 2);
    if (hi) v[18 + c] += y; else v[c] += y;
  }
  T w[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) {  // within the kept half, quarter odd, received from q ^ 1
    const T a = hi ? v[18 + c] : v[c], b = hi ? v[27 + c] : v[9 + c];
    const T y = __shfl_xor_sync(0xffffffffu, odd ? a : b, 1);
    w[c] = (odd ? b : a) + y;
  }
  if (!live) return;
  // vector stores: lanes 0-2 write sum S^00, S^01, S^11 (its 9 values, then (s, t) = (1, 1) and a
  // zero; the last 4 values of a sum are not read), lane 3 the force sums
  if (q < 3) {
    T* o = S + (long long)ELEM_SUMS * e + q * SUM_STRIDE;
    store4<T>(o, w[0], w[1], w[2], w[3]);
    store4<T>(o + 4, w[4], w[5], w[6], w[7]);
    store4<T>(o + 8, w[8], T(1), T(1), T(0));
  } else {
    T* f = S + (long long)ELEM_SUMS * ne + (long long)ELEM_FORCE * e;
    store4<T>(f, w[0], w[1], w[2], w[3]);
    store4<T>(f + 4, w[4], w[5], T(0), T(0));
  }
}

// R[dof] = base[dof] + scale * (contact force at the node) - f_ext[dof], zero where fixed, from
// the element force sums of the last element-side tangent gather: one thread per node, its
// incident elements in their list order.  The block partial sums of R^2 (each thread's six
// squares in order, then a fixed shuffle tree over the warp and over the block's warps) go to
// `part`, and the last block to finish adds them in block order into *norm2 (a fixed order
// whatever the timing); `count` (zero between launches) finds the last block.  VEC: base,
// f_ext and out are 16-byte aligned and moved as double2.
constexpr int GFE_T = 256;

XK_D double to_f64(float x) { return xk_f2d(x); }  // the conversion in integer arithmetic (the FP64 pipe is slow)
XK_D double to_f64(double x) { return x; }

template <typename T, bool VEC>
__global__ void __launch_bounds__(GFE_T) k_gather_force_elem(int n_nodes, int ne, const int32_t* __restrict__ neptr,
                                                             const int2* __restrict__ nelem, const T* __restrict__ S,
                                                             const double* __restrict__ base, double scale,
                                                             const double* __restrict__ f_ext,
                                                             const uint8_t* __restrict__ fixed,
                                                             double* __restrict__ out, double* __restrict__ part,
                                                             unsigned int* __restrict__ count,
                                                             double* __restrict__ norm2) {
  __shared__ double red[GFE_T / 32];
  __shared__ bool last;
  const int v = blockIdx.x * GFE_T + threadIdx.x;
  double sq = 0.0;
  if (v < n_nodes) {
    double r[6];
    if (base) {
      if (VEC) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const double2 x = __ldg(reinterpret_cast<const double2*>(base + 6LL * v) + i);
          r[2 * i] = x.x;
          r[2 * i + 1] = x.y;
        }
      } else {
#pragma unroll
        for (int c = 0; c < 6; ++c) r[c] = base[6LL * v + c];
      }
    } else {
#pragma unroll
      for (int c = 0; c < 6; ++c) r[c] = 0.0;
    }
    const T* F = S + (long long)ELEM_SUMS * ne;
    T acc[3] = {T(0), T(0), T(0)};
    for (int y = neptr[v]; y < neptr[v + 1]; ++y) {
      const int ex = nelem[y].x;  // (element << 1) | local index of v in it
      const T* f = F + (long long)ELEM_FORCE * (ex >> 1) + 3 * (ex & 1);
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] += f[c];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c] += scale * to_f64(acc[c]);
    if (f_ext) {
      if (VEC) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const double2 x = __ldg(reinterpret_cast<const double2*>(f_ext + 6LL * v) + i);
          r[2 * i] -= x.x;
          r[2 * i + 1] -= x.y;
        }
      } else {
#pragma unroll
        for (int c = 0; c < 6; ++c) r[c] -= f_ext[6LL * v + c];
      }
    }
    if (fixed) {
#pragma unroll
      for (int c = 0; c < 6; ++c)
        if (fixed[6LL * v + c]) r[c] = 0.0;
    }
    if (VEC) {
#pragma unroll
      for (int i = 0; i < 3; ++i) reinterpret_cast<double2*>(out + 6LL * v)[i] = make_double2(r[2 * i], r[2 * i + 1]);
    } else {
#pragma unroll
      for (int c = 0; c < 6; ++c) out[6LL * v + c] = r[c];
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) sq = fma(r[c], r[c], sq);
  }
  if (!norm2) return;  // uniform over the launch
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
  if (lane == 0) red[warp] = sq;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int w = 0; w < GFE_T / 32; ++w) b += red[w];
    part[blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(count, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double a = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += GFE_T) a += __ldcg(part + b);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if (lane == 0) red[warp] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < GFE_T / 32; ++w) t += red[w];
    *norm2 = t;
    *count = 0u;  // ready for the next launch
  }
}

template <typename T>
XK_D void load12(const T* __restrict__ p, T* v);
template <>
XK_D void load12<float>(const float* __restrict__ p, float* v) {  // p 32-byte aligned
  ldg8(p, v);
  const float4 x = __ldg(reinterpret_cast<const float4*>(p) + 2);
  v[8] = x.x; v[9] = x.y; v[10] = x.z; v[11] = x.w;
}
template <>
XK_D void load12<double>(const double* __restrict__ p, double* v) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const double2 x = __ldg(q + i);
    v[2 * i] = x.x; v[2 * i + 1] = x.y;
  }
}

// acc += one term of a block (-1: none): B and (s, t) of an element sum (s = t = 1) or of a member record
template <typename T>
XK_D void sides_term(const T* __restrict__ S, const T* __restrict__ rec, int c, T* acc) {
  if (c == -1) return;
  T v[12];
  load12<T>(c < 0 ? S + (c & 0x7fffffff) : rec + (long long)(c >> 4) * XK_REC_STRIDE_COMBINED, v);
  const int k = c < 0 ? 1 : (c >> 2) & 3, l = c < 0 ? 1 : c & 3;
  const T w = shape_c<T>(v[9], v[10], k) * shape_c<T>(v[9], v[10], l);
#pragma unroll
  for (int q = 0; q < 9; ++q) acc[q] += w * v[q];
}

// Variant "sides", step 2: one thread per block over its (at most four) inline
// terms in their sorted order: element sums, then cross contributions; the
// block values go out through shared memory so that the stores are coalesced.
constexpr int GS_T = 128;

template <typename T, int RS, int BCOL>
XK_D void add_term(const T* __restrict__ S, const T* __restrict__ rec, int code, T* acc) {
  if (code == -1) return;
  if (code < 0) {
    const T* s = S + (code & 0x7fffffff);
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q] += s[q];
  } else {
    add_contrib<T, RS, BCOL>(rec, code, acc);
  }
}

// The grid is persistent (as many CTAs per SM as are resident, each taking every gridDim.x-th tile of
// GS_T blocks): a thread loads its code of the CTA's next tile before it gathers the terms of the
// current one, so the code load's latency hides behind the term loads.
XK_D int4 sides_code(const int4* __restrict__ codes, long long nnzb, long long tile) {
  const long long b = tile * GS_T + threadIdx.x;
  return b < nnzb ? __ldcs(codes + b) : make_int4(-1, -1, -1, -1);
}

template <typename T, int RS, int BCOL>
__global__ void __launch_bounds__(GS_T, sizeof(T) == 4 ? 16 : 8) k_gather_tangent_sides(long long nnzb, const int4* __restrict__ codes,
                                                               const T* __restrict__ S, const T* __restrict__ rec,
                                                               T* __restrict__ K) {
  __shared__ __align__(16) T stage[GS_T * 9];
  const long long ntiles = (nnzb + GS_T - 1) / GS_T;
  long long tile = blockIdx.x;
  int4 cn = tile < ntiles ? sides_code(codes, nnzb, tile) : make_int4(-1, -1, -1, -1);
  for (; tile < ntiles; tile += gridDim.x) {
    const long long b0 = tile * GS_T;
    const int4 c = cn;
    if (tile + gridDim.x < ntiles) cn = sides_code(codes, nnzb, tile + gridDim.x);
    T acc[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q] = T(0);
    if (RS == XK_REC_STRIDE_COMBINED) {
      // each term is the first twelve values of its element sum or member record
      sides_term<T>(S, rec, c.x, acc);
      sides_term<T>(S, rec, c.y, acc);
      sides_term<T>(S, rec, c.z, acc);
      sides_term<T>(S, rec, c.w, acc);
    } else {
      add_term<T, RS, BCOL>(S, rec, c.x, acc);
      add_term<T, RS, BCOL>(S, rec, c.y, acc);
      add_term<T, RS, BCOL>(S, rec, c.z, acc);
      add_term<T, RS, BCOL>(S, rec, c.w, acc);
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) stage[threadIdx.x * 9 + q] = acc[q];
    __syncthreads();
    const long long rem = nnzb - b0;
    const int nv = 9 * (int)(rem < GS_T ? rem : GS_T);
    T* out = K + 9 * b0;
    if (sizeof(T) == 4 && ((uintptr_t)out & 15) == 0) {
      // 16-byte stores of the staged values (a CTA's 128 blocks are 4608 bytes)
      const int n4 = nv / 4;
      for (int v = threadIdx.x; v < n4; v += GS_T)
        reinterpret_cast<float4*>(out)[v] = reinterpret_cast<const float4*>(stage)[v];
      for (int v = 4 * n4 + threadIdx.x; v < nv; v += GS_T) out[v] = stage[v];
    } else {
      for (int v = threadIdx.x; v < nv; v += GS_T) out[v] = stage[v];
    }
    __syncthreads();  // the stage is read out before the next tile overwrites it
  }
}

// persistent grid of the sides gather: every SM's share of CTAs, or one CTA per tile when fewer
int sides_grid(long long nnzb, int per_sm) {
  const int sms = xk_sm_count();
  const long long tiles = (nnzb + GS_T - 1) / GS_T;
  const long long cap = (long long)sms * per_sm;
  return (int)(tiles < cap ? (tiles > 0 ? tiles : 1) : cap);
}


// Variant "lanes": a warp owns 32 consecutive blocks and spreads their
// contributors one per lane (32 per round); a segmented inclusive scan over
// the lanes (fixed shuffle tree, segments = blocks) sums each block's run in
// the round and the run's last lane adds it to the block's shared-memory
// accumulator.  Fewer serial steps per lane than the chunked variant below,
// more shuffles per contributor.
template <typename T, int RS, int BCOL>
__global__ void __launch_bounds__(128) k_gather_tangent_lanes(long long nnzb, const int32_t* __restrict__ bptr,
                                                             const int32_t* __restrict__ contrib,
                                                             const T* __restrict__ rec, T* __restrict__ K) {
  __shared__ T acc[4][32 * 9];
  __shared__ int ptr_s[4][33];
  const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long b0 = ((long long)blockIdx.x * 4 + wl) * 32;
  if (b0 >= nnzb) return;  // whole warp
  const int nblk = (int)((nnzb - b0) < 32 ? (nnzb - b0) : 32);
  T* A = acc[wl];
  int* P = ptr_s[wl];
#pragma unroll
  for (int q = 0; q < 9; ++q) A[q * 32 + lane] = T(0);
  P[lane] = bptr[b0 + (lane < nblk ? lane : nblk)];
  if (lane == 0) P[32] = bptr[b0 + nblk];
  __syncwarp();
  const int x0 = P[0], x1 = P[nblk];
  for (int base = x0; base < x1; base += 32) {
    const int x = base + lane;
    const bool valid = x < x1;
    int slot = 0;
    if (valid) {
      int lo = 0, hi = nblk - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P[mid] <= x) lo = mid; else hi = mid - 1;
      }
      slot = lo;
    }
    T v[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) v[q] = T(0);
    if (valid) add_contrib<T, RS, BCOL>(rec, contrib[x], v);
    const int prev_slot = __shfl_up_sync(0xffffffffu, slot, 1);
    const bool head = valid && (lane == 0 || prev_slot != slot);
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const int seg_start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        const T y = __shfl_up_sync(0xffffffffu, v[q], d);
        if (lane - d >= seg_start) v[q] += y;
      }
    }
    const int next_slot = __shfl_down_sync(0xffffffffu, slot, 1);
    const bool next_valid = __shfl_down_sync(0xffffffffu, (int)valid, 1) != 0;
    const bool tail = valid && (lane == 31 || !next_valid || next_slot != slot);
    if (tail) {
#pragma unroll
      for (int q = 0; q < 9; ++q) A[slot * 9 + q] += v[q];
    }
    __syncwarp();
  }
  for (int i = lane; i < 9 * nblk; i += 32) K[9 * b0 + i] = A[i];
}

// Variant "chunks" (default for double): Contributor counts are very uneven: 61% of the blocks of a strand have one
// contributor, a node's diagonal block up to ~36.  A warp owns 32 consecutive
// blocks and cuts their contributor list into chunks of GT_CH, one per lane
// (a round covers 32 * GT_CH contributors).  A lane sums its chunk serially;
// a block whose contributors end inside the chunk is added to the block's
// shared-memory accumulator by that lane, with the partial sums of the lanes
// before it (a segmented inclusive scan of the lanes' last partial sums over
// a fixed shuffle tree).  After the last round the warp stores its 32 x 9
// values contiguously.  Every sum is taken in a fixed order.
constexpr int GT_WARPS = 4;
constexpr int GT_CH = 4;

template <typename T, int RS, int BCOL>
__global__ void __launch_bounds__(32 * GT_WARPS) k_gather_tangent(long long nnzb, const int32_t* __restrict__ bptr,
                                                                 const int32_t* __restrict__ contrib,
                                                                 const T* __restrict__ rec, T* __restrict__ K) {
  __shared__ T acc[GT_WARPS][32 * 9];
  __shared__ int ptr_s[GT_WARPS][33];
  const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long b0 = ((long long)blockIdx.x * GT_WARPS + wl) * 32;
  if (b0 >= nnzb) return;  // whole warp
  const int nblk = (int)((nnzb - b0) < 32 ? (nnzb - b0) : 32);
  T* A = acc[wl];
  int* P = ptr_s[wl];
#pragma unroll
  for (int q = 0; q < 9; ++q) A[q * 32 + lane] = T(0);
  P[lane] = bptr[b0 + (lane < nblk ? lane : nblk)];
  if (lane == 0) P[32] = bptr[b0 + nblk];
  __syncwarp();
  const int x0 = P[0], x1 = P[nblk];
  for (int base = x0; base < x1; base += 32 * GT_CH) {
    const int c0 = base + lane * GT_CH;
    const int c1 = min(c0 + GT_CH, x1);
    const bool has = c0 < c1;
    // slot of the chunk's first contributor: last slot whose start <= c0
    int slot = 0;
    if (has) {
      int lo = 0, hi = nblk - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P[mid] <= c0) lo = mid; else hi = mid - 1;
      }
      slot = lo;
    }
    const int first_slot = slot;
    const bool first_open = has && P[slot] < c0;  // first block began before this chunk
    T part[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) part[q] = T(0);
    T head[9];  // sum over the first block's contributors in this chunk, once it is closed
    bool head_closed = false;
    for (int x = c0; x < c1; ++x) {
      while (x >= P[slot + 1]) {  // the current block ends before x: close it
        if (slot == first_slot && first_open) {
#pragma unroll
          for (int q = 0; q < 9; ++q) head[q] = part[q];
          head_closed = true;
        } else {
#pragma unroll
          for (int q = 0; q < 9; ++q) A[slot * 9 + q] += part[q];
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) part[q] = T(0);
        ++slot;
      }
      add_contrib<T, RS, BCOL>(rec, contrib[x], part);
    }
    const int last_slot = slot;
    // lanes whose last block is open at the end of the chunk pass its partial on
    // (lane 31 closes at the end of the round; the next round adds the rest)
    const bool tail_open = has && lane < 31 && c1 < P[last_slot + 1] && c1 < x1;
    // segmented inclusive scan over lanes of the last partials; a lane starts a
    // segment unless its first block continues the previous lane's last block
    const int prev_last = __shfl_up_sync(0xffffffffu, last_slot, 1);
    const bool prev_open = __shfl_up_sync(0xffffffffu, (int)tail_open, 1) != 0;
    const bool cont = lane > 0 && has && prev_open && prev_last == first_slot;
    // value entering the scan: the lane's last partial when its last block is the
    // continued first block, else its last partial alone (a new segment)
    T v[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) v[q] = part[q];
    const bool seg_head = !(cont && last_slot == first_slot && !head_closed);
    const unsigned heads = __ballot_sync(0xffffffffu, seg_head);
    const int seg_start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        const T y = __shfl_up_sync(0xffffffffu, v[q], d);
        if (lane - d >= seg_start) v[q] += y;
      }
    }
    // carry into this lane's first block = the previous lane's scanned value
    T carry[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const T y = __shfl_up_sync(0xffffffffu, v[q], 1);
      carry[q] = cont ? y : T(0);
    }
    if (has) {
      if (head_closed) {  // the first block ended inside this chunk
#pragma unroll
        for (int q = 0; q < 9; ++q) A[first_slot * 9 + q] += carry[q] + head[q];
      }
      if (!tail_open) {  // the last block ends here (or the round ends)
        if (last_slot == first_slot && !head_closed) {
#pragma unroll
          for (int q = 0; q < 9; ++q) A[last_slot * 9 + q] += v[q];  // scanned: carry + own
        } else {
#pragma unroll
          for (int q = 0; q < 9; ++q) A[last_slot * 9 + q] += part[q];
        }
      }
    }
    __syncwarp();
  }
  for (int i = lane; i < 9 * nblk; i += 32) K[9 * b0 + i] = A[i];
}

struct Scratch {
  cudaStream_t s;
  void* p[24];
  int n = 0;
  template <typename T>
  xk_status get(T** out, long long count) {
    if (n >= (int)(sizeof(p) / sizeof(p[0]))) return xk_set_error(XK_ERR_OVERFLOW, "scratch table full");
    if (count < 1) count = 1;
    cudaError_t e = cudaMallocAsync((void**)out, sizeof(T) * count, s);
    if (e != cudaSuccess) return xk_set_cuda_error(e, __FILE__, __LINE__);
    p[n++] = *out;
    return XK_OK;
  }
  ~Scratch() {
    for (int i = 0; i < n; ++i) cudaFreeAsync(p[i], s);
  }
};

#define XK_TRY(x)                 \
  do {                            \
    xk_status r__ = (x);          \
    if (r__ != XK_OK) return r__; \
  } while (0)

xk_status fetch_i64(const int64_t* dev, int64_t* host, int n, cudaStream_t st) {
  XK_CUDA(cudaMemcpyAsync(host, dev, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st));
  XK_CUDA(cudaStreamSynchronize(st));
  return XK_OK;
}

}  // namespace

extern "C" xk_status xk_contact_pattern_build(const xk_mesh* m, const xk_pairs* p, xk_contact_pattern* pat,
                                              xk_stream s) {
  if (!m || !p || !pat) return xk_set_error(XK_ERR_ARG, "xk_contact_pattern_build: null argument");
  if (!pat->inc_ptr || !pat->row_ptr) return xk_set_error(XK_ERR_ARG, "xk_contact_pattern_build: row arrays missing");
  cudaStream_t st = (cudaStream_t)s;
  const int nn = m->n_nodes;
  const long long np = p->n;
  pat->n_nodes = nn;
  Scratch S{st};
  int32_t *flag, *mpos, *cnt, *fill, *err;
  int64_t* tot;
  XK_TRY(S.get(&flag, np + 1));
  XK_TRY(S.get(&mpos, np + 1));
  XK_TRY(S.get(&cnt, nn + 1));
  XK_TRY(S.get(&fill, nn + 1));
  XK_TRY(S.get(&err, 1));
  XK_TRY(S.get(&tot, 4));
  // members and others
  k_flags<<<xk_blocks(np + 1, 256), 256, 0, st>>>(*p, flag);
  XK_CHECK_LAUNCH();
  XK_TRY(xk_exclusive_scan_i32(flag, mpos, np + 1, tot, st));
  int64_t h[4] = {0, 0, 0, 0};
  XK_TRY(fetch_i64(tot, h, 1, st));
  const long long nm = h[0];
  pat->n_members = (int32_t)nm;
  pat->n_others = (int32_t)(np - nm);
  if (nm > pat->cap_members || np - nm > pat->cap_others)
    return xk_set_error(XK_ERR_CAPACITY, "xk_contact_pattern_build: member / other-pair capacity too small");
  if (np > 0) k_split_lists<<<xk_blocks(np, 256), 256, 0, st>>>(*m, *p, mpos, pat->members, pat->member_nodes,
                                                                 pat->others);
  // node incidence of the members
  XK_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (nn + 1), st));
  if (nm > 0) k_inc_count<<<xk_blocks(nm, 256), 256, 0, st>>>(pat->member_nodes, (int)nm, cnt);
  XK_CHECK_LAUNCH();
  XK_TRY(xk_exclusive_scan_i32(cnt, pat->inc_ptr, nn + 1, nullptr, st));
  XK_CUDA(cudaMemsetAsync(fill, 0, sizeof(int32_t) * (nn + 1), st));
  if (nm > 0) k_inc_fill<<<xk_blocks(nm, 256), 256, 0, st>>>(pat->member_nodes, (int)nm, pat->inc_ptr, fill, pat->inc);
  k_segment_sort<<<xk_blocks(32LL * nn, SEG_T), SEG_T, 0, st>>>(pat->inc_ptr, nn, pat->inc);
  // block pattern rows
  XK_CUDA(cudaMemsetAsync(err, 0, sizeof(int32_t), st));
  if (nn > 0)
    k_row_cols<0><<<(unsigned)((nn + RC_WARPS - 1) / RC_WARPS), 32 * RC_WARPS, 0, st>>>(pat->member_nodes, pat->inc_ptr, pat->inc, nn, cnt, nullptr,
                                                   nullptr, nullptr, err);
  XK_CHECK_LAUNCH();
  XK_CUDA(cudaMemsetAsync(cnt + nn, 0, sizeof(int32_t), st));
  XK_TRY(xk_exclusive_scan_i32(cnt, pat->row_ptr, nn + 1, tot + 1, st));
  int32_t herr = 0;
  XK_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  XK_TRY(fetch_i64(tot, h, 2, st));
  if (herr) return xk_set_error(XK_ERR_OVERFLOW, "xk_contact_pattern_build: a node touches more than 256 contact nodes");
  const long long nb = h[1];
  pat->nnzb = nb;
  if (nb > pat->cap_blocks) return xk_set_error(XK_ERR_CAPACITY, "xk_contact_pattern_build: block capacity too small");
  if (nn > 0)
    k_row_cols<1><<<(unsigned)((nn + RC_WARPS - 1) / RC_WARPS), 32 * RC_WARPS, 0, st>>>(pat->member_nodes, pat->inc_ptr, pat->inc, nn, nullptr,
                                                   pat->row_ptr, pat->col, pat->blk_row, err);
  XK_CHECK_LAUNCH();
  // contributor lists of the blocks
  int32_t *bcnt, *bfill;
  XK_TRY(S.get(&bcnt, nb + 1));
  XK_TRY(S.get(&bfill, nb + 1));
  XK_CUDA(cudaMemsetAsync(bcnt, 0, sizeof(int32_t) * (nb + 1), st));
  if (nm > 0) k_contrib<0><<<xk_blocks(nm, 128), 128, 0, st>>>(pat->member_nodes, (int)nm, pat->row_ptr, pat->col,
                                                                bcnt, nullptr, nullptr, err);
  XK_CHECK_LAUNCH();
  XK_TRY(xk_exclusive_scan_i32(bcnt, pat->blk_ptr, nb + 1, tot + 2, st));
  XK_CUDA(cudaMemsetAsync(bfill, 0, sizeof(int32_t) * (nb + 1), st));
  if (nm > 0) k_contrib<1><<<xk_blocks(nm, 128), 128, 0, st>>>(pat->member_nodes, (int)nm, pat->row_ptr, pat->col,
                                                                bfill, pat->blk_ptr, pat->contrib, err);
  if (nb > 0) {
    int32_t *longs, *n_longs;
    XK_TRY(S.get(&longs, nb));
    XK_TRY(S.get(&n_longs, 1));
    XK_CUDA(cudaMemsetAsync(n_longs, 0, sizeof(int32_t), st));
    k_segment_sort_short<<<xk_blocks(nb, 256), 256, 0, st>>>(pat->blk_ptr, nb, pat->contrib, longs, n_longs);
    k_segment_sort_listed<<<xk_sm_count() * 8, SEG_T, 0, st>>>(pat->blk_ptr, pat->contrib, longs, n_longs);
  }
  XK_CHECK_LAUNCH();
  // lower index of the stored blocks
  pat->nnzb_full = nb;
  if (pat->low_ptr && pat->low_blk) {
    XK_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (nn + 1), st));
    if (nb > 0) k_lower_index<0><<<xk_blocks(nb, 256), 256, 0, st>>>(nb, pat->blk_row, pat->col, cnt, nullptr, nullptr);
    XK_CHECK_LAUNCH();
    XK_TRY(xk_exclusive_scan_i32(cnt, pat->low_ptr, nn + 1, tot + 3, st));
    XK_CUDA(cudaMemsetAsync(fill, 0, sizeof(int32_t) * (nn + 1), st));
    if (nb > 0)
      k_lower_index<1><<<xk_blocks(nb, 256), 256, 0, st>>>(nb, pat->blk_row, pat->col, fill, pat->low_ptr,
                                                           pat->low_blk);
    k_segment_sort<<<xk_blocks(32LL * nn, SEG_T), SEG_T, 0, st>>>(pat->low_ptr, nn, pat->low_blk);
    XK_CHECK_LAUNCH();
  }
  // the contribution and lower-index totals are read with the final synchronisation
  // element-side form (gather variant XK_GATHER_SIDES)
  const bool sides = pat->node_elem_ptr && pat->node_elem && pat->elem_ptr && pat->elem_inc && pat->bcodes;
  int32_t herr2 = 0;
  const int ne = m->n_elems;
  pat->n_elems = ne;
  pat->sides_ok = 0;
  if (sides) {
    int32_t *ecnt, *efill, *serr;
    XK_TRY(S.get(&ecnt, (long long)(ne > nn ? ne : nn) + 1));
    XK_TRY(S.get(&efill, (long long)(ne > nn ? ne : nn) + 1));
    XK_TRY(S.get(&serr, 1));
    // mesh node -> elements (mesh topology: built once per pattern and mesh)
    if (!pat->node_elem_ready) {
      XK_CUDA(cudaMemsetAsync(ecnt, 0, sizeof(int32_t) * (nn + 1), st));
      if (ne > 0) k_node_elem_count<<<xk_blocks(ne, 256), 256, 0, st>>>(*m, ecnt);
      XK_CHECK_LAUNCH();
      XK_TRY(xk_exclusive_scan_i32(ecnt, pat->node_elem_ptr, nn + 1, nullptr, st));
      XK_CUDA(cudaMemsetAsync(efill, 0, sizeof(int32_t) * (nn + 1), st));
      if (ne > 0)
        k_node_elem_fill<<<xk_blocks(ne, 256), 256, 0, st>>>(*m, pat->node_elem_ptr, efill,
                                                             reinterpret_cast<int2*>(pat->node_elem));
      k_segment_sort_pairs<<<xk_blocks(nn, 128), 128, 0, st>>>(pat->node_elem_ptr, nn,
                                                               reinterpret_cast<int2*>(pat->node_elem));
      XK_CHECK_LAUNCH();
    }
    // element -> member sides
    XK_CUDA(cudaMemsetAsync(ecnt, 0, sizeof(int32_t) * (ne + 1), st));
    if (nm > 0) k_elem_inc_count<<<xk_blocks(nm, 256), 256, 0, st>>>(*p, pat->members, (int)nm, ecnt);
    XK_CHECK_LAUNCH();
    XK_TRY(xk_exclusive_scan_i32(ecnt, pat->elem_ptr, ne + 1, nullptr, st));
    XK_CUDA(cudaMemsetAsync(efill, 0, sizeof(int32_t) * (ne + 1), st));
    if (nm > 0)
      k_elem_inc_fill<<<xk_blocks(nm, 256), 256, 0, st>>>(*p, pat->members, (int)nm, pat->elem_ptr, efill,
                                                          pat->elem_inc);
    if (ne > 0) k_segment_sort<<<xk_blocks(32LL * ne, SEG_T), SEG_T, 0, st>>>(pat->elem_ptr, ne, pat->elem_inc);
    XK_CHECK_LAUNCH();
    // inline term lists; a flag in serr (more than four terms somewhere) only disables the variant
    XK_CUDA(cudaMemsetAsync(serr, 0, sizeof(int32_t), st));
    XK_CUDA(cudaMemsetAsync(pat->bcodes, 0xff, sizeof(int32_t) * 4 * (nb > 0 ? nb : 1), st));
    if (nb > 0)
      k_side_codes<<<xk_blocks(nb, 256), 256, 0, st>>>(nb, pat->blk_row, pat->col, pat->node_elem_ptr,
                                                       reinterpret_cast<const int2*>(pat->node_elem), pat->bcodes,
                                                       bcnt, serr);
    if (nm > 0)
      k_cross_codes<<<xk_blocks(nm, 128), 128, 0, st>>>(pat->member_nodes, (int)nm, pat->row_ptr, pat->col, bcnt,
                                                        pat->bcodes, serr);
    if (nb > 0) k_sort_codes<<<xk_blocks(nb, 256), 256, 0, st>>>(nb, reinterpret_cast<int4*>(pat->bcodes));
    XK_CHECK_LAUNCH();
    XK_CUDA(cudaMemcpyAsync(&herr2, serr, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  }
  XK_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  XK_CUDA(cudaMemcpyAsync(h + 2, tot + 2, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  XK_CUDA(cudaStreamSynchronize(st));
  pat->n_contrib = h[2];
  if (pat->low_ptr && pat->low_blk) pat->nnzb_full = nb + h[3];
  if (sides) {
    pat->sides_ok = herr2 ? 0 : 1;
    pat->node_elem_ready = 1;
  }
  if (herr) return xk_set_error(XK_ERR_OVERFLOW, "xk_contact_pattern_build: inconsistent block pattern");
  return XK_OK;
}

static bool aligned32(const void* p) { return ((uintptr_t)p & 31) == 0; }

static xk_status rec_columns(int out_mode, int which, bool tangent, int* c1, int* c2) {
  *c2 = -1;
  if (out_mode == XK_OUT_COMBINED) {
    if (which != XK_WHICH_COMBINED) return xk_set_error(XK_ERR_ARG, "combined records hold only combined values");
    *c1 = tangent ? XK_REC_B : XK_REC_V;
    return XK_OK;
  }
  if (out_mode != XK_OUT_SPLIT) return xk_set_error(XK_ERR_ARG, "out_mode");
  if (tangent) {
    if (which == XK_WHICH_NORMAL) *c1 = 8;
    else if (which == XK_WHICH_FRICTION) *c1 = 17;
    else return xk_set_error(XK_ERR_ARG, "split tangent records need which = normal or friction");
  } else {
    if (which == XK_WHICH_NORMAL) *c1 = 2;
    else if (which == XK_WHICH_FRICTION) *c1 = 5;
    else { *c1 = 2; *c2 = 5; }
  }
  return XK_OK;
}

extern "C" xk_status xk_contact_gather_force(const xk_contact_pattern* pat, const void* rec, int precision,
                                             int out_mode, int which, const double* base, double scale,
                                             const double* f_ext, const uint8_t* fixed, double* out, double* norm2,
                                             xk_stream s) {
  if (!pat || !out) return xk_set_error(XK_ERR_ARG, "xk_contact_gather_force: null argument");
  int c1, c2;
  XK_TRY(rec_columns(out_mode, which, false, &c1, &c2));
  const int rs = out_mode == XK_OUT_COMBINED ? XK_REC_STRIDE_COMBINED : XK_REC_STRIDE_SPLIT;
  const int stc = out_mode == XK_OUT_COMBINED ? XK_REC_S : 0;
  const bool use = pat->n_members > 0 && rec;
  const int32_t* ptr = use ? pat->inc_ptr : nullptr;
  const int32_t* inc = use ? pat->inc : nullptr;
  cudaStream_t st = (cudaStream_t)s;
  const int nn = pat->n_nodes;
  if (nn > 0) {
    if (precision == XK_FP64)
      k_gather_force<double><<<xk_blocks((long long)GF_LANES * nn, 128), 128, 0, st>>>(nn, ptr, inc, (const double*)rec, rs, stc, c1, c2,
                                                                         base, scale, f_ext, fixed, out);
    else if (precision == XK_MIXED)
      k_gather_force<float><<<xk_blocks((long long)GF_LANES * nn, 128), 128, 0, st>>>(nn, ptr, inc, (const float*)rec, rs, stc, c1, c2,
                                                                        base, scale, f_ext, fixed, out);
    else
      return xk_set_error(XK_ERR_ARG, "xk_contact_gather_force: precision");
    XK_CHECK_LAUNCH();
  }
  if (norm2) return xk_sumsq_into(out, 6LL * nn, norm2, st);
  return XK_OK;
}

extern "C" xk_status xk_contact_gather_force_elem(const xk_contact_pattern* pat, int precision, const double* base,
                                                  double scale, const double* f_ext, const uint8_t* fixed,
                                                  double* out, double* norm2, xk_stream s) {
  if (!pat || !out) return xk_set_error(XK_ERR_ARG, "xk_contact_gather_force_elem: null argument");
  if (!pat->node_elem_ptr || !pat->node_elem || !pat->elem_sums || (norm2 && !pat->norm_scratch))
    return xk_set_error(XK_ERR_ARG, "xk_contact_gather_force_elem: the element-side pattern was not built");
  if (precision != XK_FP64 && precision != XK_MIXED)
    return xk_set_error(XK_ERR_ARG, "xk_contact_gather_force_elem: precision");
  const int nn = pat->n_nodes, ne = (int)pat->n_elems;
  if (nn <= 0) {
    if (norm2) XK_CUDA(cudaMemsetAsync(norm2, 0, sizeof(double), (cudaStream_t)s));
    return XK_OK;
  }
  const int nb = xk_blocks(nn, GFE_T);  // <= (6 n_nodes + 255) / 256, the partial sums of norm_scratch
  double* part = pat->norm_scratch;
  unsigned int* count = part ? reinterpret_cast<unsigned int*>(part + nb) : nullptr;
  const int2* nelem = reinterpret_cast<const int2*>(pat->node_elem);
  const bool vec = ((uintptr_t)base & 15) == 0 && ((uintptr_t)f_ext & 15) == 0 && ((uintptr_t)out & 15) == 0;
  cudaStream_t st = (cudaStream_t)s;
#define XK_GFE(TT, VV)                                                                                           \
  k_gather_force_elem<TT, VV><<<nb, GFE_T, 0, st>>>(nn, ne, pat->node_elem_ptr, nelem, (const TT*)pat->elem_sums, \
                                                    base, scale, f_ext, fixed, out, part, count, norm2)
  if (precision == XK_FP64) {
    if (vec) XK_GFE(double, true); else XK_GFE(double, false);
  } else {
    if (vec) XK_GFE(float, true); else XK_GFE(float, false);
  }
#undef XK_GFE
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_contact_gather_tangent(const xk_contact_pattern* pat, const void* rec, int precision,
                                               int out_mode, int which, int variant, void* Kc_vals, xk_stream s) {
  if (!pat || !rec || !Kc_vals) return xk_set_error(XK_ERR_ARG, "xk_contact_gather_tangent: null argument");
  int c1, c2;
  XK_TRY(rec_columns(out_mode, which, true, &c1, &c2));
  if (variant < 0 || variant > XK_GATHER_SIDES_BLOCKS)
    return xk_set_error(XK_ERR_ARG, "xk_contact_gather_tangent: variant");
  const bool sides = variant >= XK_GATHER_SIDES;
  const bool sums = variant != XK_GATHER_SIDES_BLOCKS, blocks = variant != XK_GATHER_SIDES_SUMS;
  if (sides && out_mode == XK_OUT_COMBINED && !(aligned32(rec) && aligned32(pat->elem_sums)))
    return xk_set_error(XK_ERR_ARG, "xk_contact_gather_tangent: rec and elem_sums must be 32-byte aligned");
  if (sides && !(pat->elem_ptr && pat->elem_inc && pat->bcodes && pat->elem_sums && pat->sides_ok == 1))
    return xk_set_error(XK_ERR_ARG, "xk_contact_gather_tangent: the element-side pattern was not built");
  if (pat->nnzb == 0) return XK_OK;
  cudaStream_t st = (cudaStream_t)s;
  const int nb = xk_blocks((pat->nnzb + 31) / 32, GT_WARPS);
  const bool comb = out_mode == XK_OUT_COMBINED;
  // variant: 0 default (chunks for double, lanes for float), 1 lanes, 2 chunks, 3 element sides
  const bool chunks = variant == 2 || (variant == 0 && precision == XK_FP64);
  const int ne = (int)pat->n_elems;
#define XK_GT(TT, RSV, BC)                                                                                   \
  do {                                                                                                      \
    if (sides) {                                                                                            \
      if (sums && ne > 0 && RSV == XK_REC_STRIDE_COMBINED)                                                  \
        k_elem_sums_rec<TT><<<xk_blocks(4LL * ne, 128), 128, 0, st>>>(ne, pat->elem_ptr, pat->elem_inc,     \
                                                                (const TT*)rec, (TT*)pat->elem_sums);       \
      else if (sums && ne > 0)                                                                              \
        k_elem_sums<TT, RSV, BC><<<xk_blocks(9LL * ne, 256), 256, 0, st>>>(ne, pat->elem_ptr, pat->elem_inc,   \
                                                                           (const TT*)rec, (TT*)pat->elem_sums); \
      if (blocks)                                                                                           \
        k_gather_tangent_sides<TT, RSV, BC><<<sides_grid(pat->nnzb, pat->sides_per_sm > 0 ? pat->sides_per_sm : (sizeof(TT) == 4 ? 16 : 8)), GS_T, 0, st>>>( \
            pat->nnzb, reinterpret_cast<const int4*>(pat->bcodes), (const TT*)pat->elem_sums, (const TT*)rec,  \
            (TT*)Kc_vals);                                                                                  \
    } else if (chunks)                                                                                      \
      k_gather_tangent<TT, RSV, BC><<<nb, 32 * GT_WARPS, 0, st>>>(pat->nnzb, pat->blk_ptr, pat->contrib,     \
                                                                  (const TT*)rec, (TT*)Kc_vals);            \
    else                                                                                                    \
      k_gather_tangent_lanes<TT, RSV, BC><<<xk_blocks((pat->nnzb + 31) / 32, 4), 128, 0, st>>>(             \
          pat->nnzb, pat->blk_ptr, pat->contrib, (const TT*)rec, (TT*)Kc_vals);                             \
  } while (0)
  if (precision == XK_FP64) {
    if (comb) XK_GT(double, 16, XK_REC_B);
    else if (c1 == 8) XK_GT(double, 32, 8);
    else XK_GT(double, 32, 17);
  } else if (precision == XK_MIXED) {
    if (comb) XK_GT(float, 16, XK_REC_B);
    else if (c1 == 8) XK_GT(float, 32, 8);
    else XK_GT(float, 32, 17);
  } else {
    return xk_set_error(XK_ERR_ARG, "xk_contact_gather_tangent: precision");
  }
#undef XK_GT
  XK_CHECK_LAUNCH();
  return XK_OK;
}
