// Broadphase and pair-list update.
//
// The reference bins AABBs into a hash grid (xkep_cae/contact/_broadphase.py:52-87)
// and keeps the pairs whose closed AABBs overlap (:93-96); its output is the
// set of all overlapping pairs, whatever the cell size.  Here every segment is
// binned once, by the cell of its box's lower corner (counting sort by cell, each cell's entries then
// in ascending order).
// A box j can overlap box i only if its lower corner lies in [lo_i - E, hi_i]
// per axis, E the largest extent of any box on that axis, so a warp per
// segment i walks the cells of that range (32 cells a batch) and tests every
// entry j > i (found in each cell by a binary search): screened on float boxes rounded outward, tested on the exact
// double AABBs, filtered, compacted with ballot/popc into a fixed-size slot list
// of the segment.  Each pair is found once, from its lower-numbered segment, in
// a single walk: a second kernel sorts each slot list and applies the midpoint
// prescreen (whose margin is a mean over all candidates), a third writes the
// kept pairs out in (i, j) order.  A slot list that overflows is detected at the
// end and the walk is repeated with longer lists.  Filters follow
// DetectCandidatesProcess (_manager_process.py:200-217,260-286).
#include <atomic>
#include <cstdio>

#include "xk_common.cuh"

namespace {

constexpr int BP_T = 128;  // 4 warps per block, one warp per segment

struct Grid {
  double origin[3];
  double cell;
  int dims[3];
  int pad;
  double emax[3];  // largest box extent on each axis
};

XK_D unsigned long long enc_min(double x) {  // order-preserving map of doubles to u64
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
XK_D double dec_min(unsigned long long k) {
  unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

// box: the FP64 boxes, six doubles per segment (lower corner, upper corner); boxf: the same boxes in
// float, rounded outward (lower corner down, upper corner up), as two float4 per segment (32 bytes): a
// conservative screen for the sweep, which then tests the FP64 boxes.  mid: per segment its midpoint and
// half length in the operation order of the midpoint prescreen (_manager_process.py:265-272), so that
// the prescreen of a pair reads these 32 bytes of each segment and gives the same values.
__global__ void k_aabb(xk_mesh m, const double* __restrict__ u, double margin, double* __restrict__ box,
                       float4* __restrict__ boxf, double4_32a* __restrict__ mid, unsigned long long* __restrict__ ext,
                       double* __restrict__ ext_sum) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long lmin[3] = {~0ull, ~0ull, ~0ull}, lmax[3] = {0ull, 0ull, 0ull}, lax[3] = {0ull, 0ull, 0ull};
  double msum = 0.0;
  if (e < m.n_elems) {
    int a = m.conn[2 * e], b = m.conn[2 * e + 1];
    const double ex = xadd(m.radii[e], margin);
    double mx = 0.0;
    float lf[3], hf[3];
    double ma[3], da[3];
    for (int c = 0; c < 3; ++c) {
      double x0 = u ? xadd(m.X[3LL * a + c], u[6LL * a + c]) : m.X[3LL * a + c];
      double x1 = u ? xadd(m.X[3LL * b + c], u[6LL * b + c]) : m.X[3LL * b + c];
      ma[c] = xmul(0.5, xadd(x0, x1));
      da[c] = xsub(x1, x0);
      double lo = xsub(x0 < x1 ? x0 : x1, ex);
      double hi = xadd(x0 < x1 ? x1 : x0, ex);
      box[6LL * e + c] = lo;
      box[6LL * e + 3 + c] = hi;
      lf[c] = __double2float_rd(lo);
      hf[c] = __double2float_ru(hi);
      lmin[c] = enc_min(lo);
      lmax[c] = enc_min(hi);
      const double extc = hi - lo;  // >= 0: the bit patterns order as the values
      lax[c] = (unsigned long long)__double_as_longlong(extc);
      mx = fmax(mx, extc);
    }
    // the spare fourth word carries the element's layer (-1 without layers), read by the walk's filter
    boxf[2LL * e] = make_float4(lf[0], lf[1], lf[2], __int_as_float(m.layer ? m.layer[e] : -1));
    boxf[2LL * e + 1] = make_float4(hf[0], hf[1], hf[2], 0.f);
    double4_32a me;
    me.x = ma[0];
    me.y = ma[1];
    me.z = ma[2];
    me.w = xmul(0.5, xsqrt(xdot_seq(da, da)));
    mid[e] = me;
    msum = mx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    for (int c = 0; c < 3; ++c) {
      unsigned long long y = __shfl_down_sync(0xffffffffu, lmin[c], o);
      lmin[c] = y < lmin[c] ? y : lmin[c];
      y = __shfl_down_sync(0xffffffffu, lmax[c], o);
      lmax[c] = y > lmax[c] ? y : lmax[c];
      y = __shfl_down_sync(0xffffffffu, lax[c], o);
      lax[c] = y > lax[c] ? y : lax[c];
    }
    msum += __shfl_down_sync(0xffffffffu, msum, o);
  }
  if ((threadIdx.x & 31) == 0) {
    for (int c = 0; c < 3; ++c) {
      atomicMin(&ext[1 + c], lmin[c]);
      atomicMax(&ext[4 + c], lmax[c]);
      atomicMax(&ext[9 + c], lax[c]);
    }
    atomicAdd(ext_sum, msum);  // the cell size only sets the work, not the result: any order will do
  }
}
// the grid over the boxes' bounding box: cells of cell_size, or (cell_size <= 0) of AUTO_CELL times the
// mean of each box's largest extent; coarsened while it would have more than cap_cells cells
constexpr double AUTO_CELL = 0.5;
__global__ void k_grid(const unsigned long long* __restrict__ ext, const double* __restrict__ ext_sum, long long ne,
                       long long cap_cells, double cell_size, Grid* g) {
  double mx = *ext_sum / (double)ne;
  double lo[3], hi[3];
  for (int c = 0; c < 3; ++c) {
    lo[c] = dec_min(ext[1 + c]);
    hi[c] = dec_min(ext[4 + c]);
  }
  double cell = cell_size > 0.0 ? cell_size : AUTO_CELL * mx * (1.0 + 1e-6) + 1e-300;
  long long tot;
  int dims[3];
  for (int it = 0; it < 200; ++it) {
    tot = 1;
    for (int c = 0; c < 3; ++c) {
      double n = floor((hi[c] - lo[c]) / cell) + 1.0;
      if (n > 2097151.0) n = 2097151.0;
      dims[c] = (int)n;
      tot *= dims[c];
    }
    if (tot <= cap_cells) break;
    cell *= 1.25;
  }
  for (int c = 0; c < 3; ++c) {
    g->origin[c] = lo[c];
    g->dims[c] = dims[c];
  }
  g->cell = cell;
  for (int c = 0; c < 3; ++c) g->emax[c] = __longlong_as_double((long long)ext[9 + c]);
}

XK_D void cell_of(const Grid& g, double lo0, double lo1, double lo2, int* c) {
  const double l[3] = {lo0, lo1, lo2};
  for (int k = 0; k < 3; ++k) {
    double f = floor((l[k] - g.origin[k]) / g.cell);
    int ci = (int)f;
    c[k] = ci < 0 ? 0 : (ci >= g.dims[k] ? g.dims[k] - 1 : ci);
  }
}

// per-cell counts of the segments binned by the cell of their box's lower corner
__global__ void k_cell_count(const double* __restrict__ box, long long ne, const Grid* __restrict__ gp,
                             int32_t* __restrict__ ecell, int32_t* __restrict__ ccnt) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const Grid g = *gp;
  int c[3];
  cell_of(g, box[6 * e], box[6 * e + 1], box[6 * e + 2], c);
  const int lin = (int)(((long long)c[2] * g.dims[1] + c[1]) * g.dims[0] + c[0]);
  ecell[e] = lin;
  atomicAdd(&ccnt[lin], 1);
}

// counting sort of the segments by cell, then each cell's entries in ascending order (a thread per cell;
// cells of more than CELL_SORTED entries are left as they are)
__global__ void k_cell_scatter(long long ne, const int32_t* __restrict__ ecell, const int32_t* __restrict__ cstart,
                               int32_t* __restrict__ cfill, int32_t* __restrict__ segs) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int c = ecell[e];
  segs[cstart[c] + atomicAdd(&cfill[c], 1)] = (int32_t)e;
}
constexpr int CELL_SORTED = 64;  // cells with more entries stay unsorted (insertion sort by one thread)
__global__ void k_cell_sort(long long ncell, const int32_t* __restrict__ cstart, int32_t* __restrict__ segs) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int lo = cstart[c], hi = cstart[c + 1];
  if (hi - lo > CELL_SORTED) return;
  for (int x = lo + 1; x < hi; ++x) {
    const int key = segs[x];
    int y = x - 1;
    while (y >= lo && segs[y] > key) { segs[y + 1] = segs[y]; --y; }
    segs[y + 1] = key;
  }
}

// the neighbouring floats above and below x (finite x): the outward-rounded float bounds lf <= lo, hf >= hi
// of a box satisfy lo <= up1(lf) and hi >= dn1(hf), so boxes whose up1/dn1-shrunk float bounds overlap
// certainly overlap in FP64 as well
XK_D float up1(float x) {
  const int b = __float_as_int(x);
  return __int_as_float(x == 0.f ? 1 : (x > 0.f ? b + 1 : b - 1));
}
XK_D float dn1(float x) {
  const int b = __float_as_int(x);
  return __int_as_float(x == 0.f ? (int)0x80000001 : (x > 0.f ? b - 1 : b + 1));
}

// the FP64 boxes of i (registers) and j (six doubles at box + 6 j, 16-byte aligned) overlap, closed
XK_D bool overlap(const double (&bi)[6], const double* __restrict__ box, int j) {
  const double2* bj = reinterpret_cast<const double2*>(box + 6LL * j);
  const double2 p = __ldg(bj), q = __ldg(bj + 1), r = __ldg(bj + 2);  // lo x,y | lo z, hi x | hi y,z
  return bi[0] <= q.y && p.x <= bi[3] && bi[1] <= r.x && p.y <= bi[4] && bi[2] <= r.y && q.x <= bi[5];
}

// A warp per segment i.  The cells that can hold the lower corner of a box overlapping box i, those
// of [lo_i - E, hi_i] (E per axis the largest extent of any box, widened by a relative 1e-12 against
// rounding), are taken 32 at a time: lane l reads cell l's entry range, a warp scan lays the ranges
// out as one list, and the warp walks it 32 entries at a time, each lane finding its entry's cell
// by a binary search over the offsets held in the lanes.  An entry j > i is screened on the
// outward-rounded float boxes (which can never reject an FP64 overlap), tested on the FP64 boxes,
// then the shared-node and same-layer filters apply and hits are compacted with ballot/popc into
// segment i's slot list (the first `cap` of them; cnt[i] counts them all).  Also per segment: the sum
// of r_i + r_j over its kept candidates (each lane sums its own entries in walk order, then a fixed
// butterfly: rsum[i], for the prescreen margin), the raw overlap count and the longest list.
__global__ void __launch_bounds__(BP_T, 7) k_sweep(xk_mesh m, const double* __restrict__ box,
                                                const float4* __restrict__ boxf, const Grid* __restrict__ gp,
                                                const int32_t* __restrict__ segs, const int32_t* __restrict__ cstart,
                                                int excl_shared, int excl_layer, int cap, int32_t* __restrict__ slot,
                                                int32_t* __restrict__ cnt, double* __restrict__ rsum,
                                                unsigned long long* __restrict__ raw_total,
                                                int32_t* __restrict__ max_cnt) {
  const long long ne = m.n_elems;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= ne) return;
  const Grid g = *gp;
  const int i = (int)w;
  double bi[6];
  for (int c = 0; c < 6; ++c) bi[c] = box[6LL * i + c];
  int c0[3], c1[3];
  {
    double lw[3];
    for (int c = 0; c < 3; ++c) lw[c] = xsub(xsub(bi[c], g.emax[c]), 1e-12 * (fabs(bi[c]) + g.emax[c]));
    cell_of(g, lw[0], lw[1], lw[2], c0);
    cell_of(g, bi[3], bi[4], bi[5], c1);
  }
  const int sx = c1[0] - c0[0] + 1, sy = c1[1] - c0[1] + 1, sz = c1[2] - c0[2] + 1;
  const int ncell = sx * sy * sz;
  const int ia = m.conn[2 * i], ib = m.conn[2 * i + 1];
  const int li = (excl_layer && m.layer) ? m.layer[i] : -1;
  const float4 il = boxf[2LL * i], ih = boxf[2LL * i + 1];
  const float iux = up1(il.x), iuy = up1(il.y), iuz = up1(il.z);  // box i shrunk to within its FP64 bounds
  const float idx_ = dn1(ih.x), idy = dn1(ih.y), idz = dn1(ih.z);
  const double ri = m.radii[i];
  int32_t* const my = slot + (long long)i * cap;
  int n_raw = 0, n_keep = 0;
  double rs = 0.0;
  for (int cb = 0; cb < ncell; cb += 32) {
    // this lane's cell of the batch and its entry range
    int s0 = 0, n0 = 0;
    const int q0 = cb + lane;
    if (q0 < ncell) {
      const int x = c0[0] + q0 % sx, y = c0[1] + (q0 / sx) % sy, z = c0[2] + q0 / (sx * sy);
      const int lin = (int)(((long long)z * g.dims[1] + y) * g.dims[0] + x);
      s0 = cstart[lin];
      const int e0 = cstart[lin + 1];
      // a cell of at most CELL_SORTED entries holds them in ascending order: only those past i can pair
      // with it (each pair is taken from its lower-numbered segment); a larger one is walked whole
      int lo = s0, hi = e0;
      if (e0 - s0 <= CELL_SORTED)
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (segs[mid] <= i) lo = mid + 1; else hi = mid;
        }
      s0 = lo;
      n0 = e0 - lo;
    }
    int incl = n0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int pre = incl - n0;
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int nq = (ncell - cb) < 32 ? (ncell - cb) : 32;
    // two entries per lane and pass (f and f + 32), their loads issued together: half the dependent
    // round trips of one entry per lane; each lane still meets its entries in increasing f
    auto entry = [&](int f) {  // the segment at list position f of the batch, or -1
      int q = 0;  // the last cell q of the batch with pre_q <= f (cells without entries share their successor's offset)
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int cand = q + step;
        const int pc = __shfl_sync(0xffffffffu, pre, cand < nq ? cand : nq - 1);
        if (cand < nq && pc <= f) q = cand;
      }
      const int sq = __shfl_sync(0xffffffffu, s0, q);
      const int pq = __shfl_sync(0xffffffffu, pre, q);
      return f < total ? segs[sq + (f - pq)] : -1;
    };
    const int2* conn2 = reinterpret_cast<const int2*>(m.conn);
    // an outward float overlap is an FP64 overlap when the boxes shrunk by one float step still overlap;
    // only the rare pair between the two takes the FP64 boxes
    auto hit_of = [&](int j, const float4& jl, const float4& jh) {
      if (!(il.x <= jh.x && jl.x <= ih.x && il.y <= jh.y && jl.y <= ih.y && il.z <= jh.z && jl.z <= ih.z))
        return false;
      const bool sure = iux <= dn1(jh.x) && up1(jl.x) <= idx_ && iuy <= dn1(jh.y) && up1(jl.y) <= idy &&
                        iuz <= dn1(jh.z) && up1(jl.z) <= idz;
      return sure || overlap(bi, box, j);
    };
    for (int f0 = 0; f0 < total; f0 += 64) {
      const int jA = entry(f0 + lane), jB = entry(f0 + 32 + lane);
      const bool nearA = jA > i, nearB = jB > i;
      float4 al = make_float4(0.f, 0.f, 0.f, 0.f), ah = al, bl = al, bh = al;
      int2 ca = make_int2(-1, -1), cb2 = ca;
      if (nearA) { al = __ldg(boxf + 2LL * jA); ah = __ldg(boxf + 2LL * jA + 1); ca = __ldg(conn2 + jA); }
      if (nearB) { bl = __ldg(boxf + 2LL * jB); bh = __ldg(boxf + 2LL * jB + 1); cb2 = __ldg(conn2 + jB); }
      const bool hitA = nearA && hit_of(jA, al, ah), hitB = nearB && hit_of(jB, bl, bh);
      bool keptA = hitA, keptB = hitB;
      if (excl_shared) {
        if (ia == ca.x || ia == ca.y || ib == ca.x || ib == ca.y) keptA = false;
        if (ia == cb2.x || ia == cb2.y || ib == cb2.x || ib == cb2.y) keptB = false;
      }
      if (li >= 0) {
        if (__float_as_int(al.w) == li) keptA = false;
        if (__float_as_int(bl.w) == li) keptB = false;
      }
      n_raw += __popc(__ballot_sync(0xffffffffu, hitA)) + __popc(__ballot_sync(0xffffffffu, hitB));
      const unsigned balA = __ballot_sync(0xffffffffu, keptA), balB = __ballot_sync(0xffffffffu, keptB);
      const unsigned below = (1u << lane) - 1u;
      if (keptA) {
        rs = xadd(rs, xadd(ri, m.radii[jA]));  // this lane's entries, in walk order
        const int at = n_keep + __popc(balA & below);
        if (at < cap) my[at] = jA;
      }
      n_keep += __popc(balA);
      if (keptB) {
        rs = xadd(rs, xadd(ri, m.radii[jB]));
        const int at = n_keep + __popc(balB & below);
        if (at < cap) my[at] = jB;
      }
      n_keep += __popc(balB);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) rs += __shfl_xor_sync(0xffffffffu, rs, o);  // fixed butterfly order
  if (lane == 0) {
    cnt[i] = n_keep;
    rsum[i] = rs;
    atomicAdd(raw_total, (unsigned long long)n_raw);
    atomicMax(max_cnt, n_keep);
  }
}

constexpr int RED_BLOCKS = 304, RED_T = 256;

// prescreen margin: mean(r_a + r_b) / 2 over the candidates after the shared-node and same-layer
// filters (_manager_process.py:275-279), from the per-segment sums, in a fixed order
__global__ void k_radsum_partial(const double* __restrict__ rsum, long long ne, double* __restrict__ part) {
  __shared__ double sm[RED_T];
  double acc = 0.0;
  for (long long k = (long long)blockIdx.x * RED_T + threadIdx.x; k < ne; k += (long long)RED_BLOCKS * RED_T)
    acc += rsum[k];
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int w = RED_T / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

__global__ void k_margin(const double* __restrict__ part, const int64_t* __restrict__ n, double fixed,
                         double* __restrict__ out) {
  if (fixed > 0.0) { *out = fixed; return; }
  double s = 0.0;
  for (int b = 0; b < RED_BLOCKS; ++b) s += part[b];
  *out = *n > 0 ? xmul(xdiv(s, (double)*n), 0.5) : 0.0;
}

// Midpoint prescreen of DetectCandidatesProcess (_manager_process.py:260-286) for the pair (i, j), from
// the segments' midpoints and half lengths: keep when max(0, |m_i - m_j| - h_i - h_j) <= r_i + r_j +
// extra, in the reference's operation order.
XK_D bool midpoint_keep(const double4_32a a, const double4_32a b, double ra, double rb, double extra) {
  const double dm[3] = {xsub(a.x, b.x), xsub(a.y, b.y), xsub(a.z, b.z)};
  const double md = xsqrt(xdot_seq(dm, dm));
  double mp = xsub(xsub(md, a.w), b.w);
  mp = (mp > 0.0 || mp != mp) ? mp : 0.0;
  return mp <= xadd(xadd(ra, rb), extra);
}

// The same decision with a float screen first: the separation |m_i - m_j| in float (from the exact double
// differences) against the threshold r_i + r_j + extra + h_i + h_j decides every pair farther than a
// relative 1e-5 from it (float rounding of the separation stays below 1e-6 relative); the rest take the
// exact routine, so the decision is the exact one.
XK_D bool midpoint_keep_fast(const double4_32a a, const double4_32a b, double ra, double rb, double extra) {
  const float dx = (float)xsub(a.x, b.x), dy = (float)xsub(a.y, b.y), dz = (float)xsub(a.z, b.z);
  const float md = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
  const float thr = (float)(ra + rb + extra + a.w + b.w);
  if (md < __fmul_rn(thr, 0.99999f)) return true;
  if (md > __fmul_rn(thr, 1.00001f)) return false;
  return midpoint_keep(a, b, ra, rb, extra);
}

// A warp per segment: its slot list sorted by j (a rank sort; the j are distinct), the prescreen
// applied (extra null: none), written to srt as j (kept) or ~j (dropped); cnt2[i] = kept count.
__global__ void __launch_bounds__(BP_T) k_slots_rank(xk_mesh m, const double4_32a* __restrict__ mid,
                                                     const int32_t* __restrict__ slot, const int32_t* __restrict__ cnt,
                                                     int cap, const double* __restrict__ extra,
                                                     int32_t* __restrict__ srt, int32_t* __restrict__ cnt2) {
  const long long ne = m.n_elems;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= ne) return;
  const int i = (int)w;
  const int n = cnt[i] < cap ? cnt[i] : cap;
  const int32_t* const my = slot + (long long)i * cap;
  int32_t* const out = srt + (long long)i * cap;
  const double4_32a mi = mid[i];
  const double ri = m.radii[i];
  const double ex = extra ? *extra : 0.0;
  int kept = 0;
  if (n <= 64) {  // two entries per lane, ranked by shuffle-broadcast comparisons
    const int v0 = lane < n ? my[lane] : 0x7fffffff;
    const int v1 = lane + 32 < n ? my[lane + 32] : 0x7fffffff;
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
    if (lane < n) {
      const bool k = !extra || midpoint_keep_fast(mi, mid[v0], ri, m.radii[v0], ex);
      out[r0] = k ? v0 : ~v0;
      kept += k;
    }
    if (lane + 32 < n) {
      const bool k = !extra || midpoint_keep_fast(mi, mid[v1], ri, m.radii[v1], ex);
      out[r1] = k ? v1 : ~v1;
      kept += k;
    }
  } else for (int l = lane; l < n; l += 32) {
    const int v = my[l];
    int r = 0;
    for (int q = 0; q < n; ++q) r += my[q] < v;
    const bool k = !extra || midpoint_keep_fast(mi, mid[v], ri, m.radii[v], ex);
    out[r] = k ? v : ~v;
    kept += k;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
  if (lane == 0) cnt2[i] = kept;
}

// A warp per segment: its kept pairs, in order, at off2[i] of out (rows (i, j); at most cap_out rows).
__global__ void __launch_bounds__(BP_T) k_slots_emit(long long ne, const int32_t* __restrict__ srt,
                                                     const int32_t* __restrict__ cnt, int cap,
                                                     const int32_t* __restrict__ off2, long long cap_out,
                                                     int32_t* __restrict__ out) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= ne) return;
  const int i = (int)w;
  const int n = cnt[i] < cap ? cnt[i] : cap;
  const int32_t* const my = srt + (long long)i * cap;
  long long at = off2[i];
  for (int l0 = 0; l0 < n; l0 += 32) {
    const int l = l0 + lane;
    const int v = l < n ? my[l] : -1;
    const unsigned bal = __ballot_sync(0xffffffffu, v >= 0);
    const long long d = at + __popc(bal & ((1u << lane) - 1u));
    if (v >= 0 && d >= 0 && d < cap_out) {
      out[2 * d] = i;
      out[2 * d + 1] = v;
    }
    at += __popc(bal);
  }
}

// ------------------------------------------------------------------------- merge


// start[s] = the first row of a list sorted by (a, b) whose a >= s, s in [0, ne] (a binary search per s; the
// rows' a values are read at stride S: 1 for a table, 2 for (a, b) rows)
template <int S>
__global__ void k_seg_start(const int32_t* __restrict__ a, long long n, long long ne, int32_t* __restrict__ start) {
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s > ne) return;
  long long lo = 0, hi = n;
  while (lo < hi) {
    long long mid = (lo + hi) >> 1;
    if (a[S * mid] < s) lo = mid + 1; else hi = mid;
  }
  start[s] = (int32_t)lo;
}

// the first row in [lo, hi) of a list sorted by b within one a whose b >= key
XK_D long long lower_bound_b(const int32_t* __restrict__ b, int S, long long lo, long long hi, int key) {
  while (lo < hi) {
    long long mid = (lo + hi) >> 1;
    if (b[S * mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

XK_D long long lower_bound_old(const xk_pairs& p, const int32_t* __restrict__ start, int a, int b) {
  return lower_bound_b(p.eb, 1, start[a], start[a + 1], b);
}
XK_D long long lower_bound_cand(const int32_t* c, const int32_t* __restrict__ start, int a, int b) {
  return lower_bound_b(c + 1, 2, start[a], start[a + 1], b);
}

XK_D void copy_state(const xk_pairs& a, long long i, xk_pairs& b, long long j) {
  const long long ca = a.cap, cb = b.cap;
  b.ea[j] = a.ea[i];
  b.eb[j] = a.eb[i];
  b.s[j] = a.s[i];
  b.t[j] = a.t[i];
  b.gap[j] = a.gap[i];
  for (int c = 0; c < 3; ++c) {
    b.normal[c * cb + j] = a.normal[c * ca + i];
    b.t1[c * cb + j] = a.t1[c * ca + i];
    b.t2[c * cb + j] = a.t2[c * ca + i];
  }
  b.lambda_n[j] = a.lambda_n[i];
  b.k_pen[j] = a.k_pen[i];
  b.k_t[j] = a.k_t[i];
  b.p_n[j] = a.p_n[i];
  b.z_t[j] = a.z_t[i];
  b.z_t[cb + j] = a.z_t[ca + i];
  b.q_trial_norm[j] = a.q_trial_norm[i];
  b.dissipation[j] = a.dissipation[i];
  b.status[j] = a.status[i];
  b.stick[j] = a.stick[i];
  if (b.coat_cc) {  // coated wires: the coating state travels with the pair (fresh if the source has none)
    const bool has = a.coat_cc != nullptr;
    b.coat_cc[j] = has ? a.coat_cc[i] : 0.0;
    b.coat_cc_prev[j] = has ? a.coat_cc_prev[i] : 0.0;
    b.coat_z_t[j] = has ? a.coat_z_t[i] : 0.0;
    b.coat_z_t[cb + j] = has ? a.coat_z_t[ca + i] : 0.0;
    b.coat_qtn[j] = has ? a.coat_qtn[i] : 0.0;
    b.coat_diss[j] = has ? a.coat_diss[i] : 0.0;
    b.coat_stick[j] = has ? a.coat_stick[i] : 1;
  }
}

// r[o] = 1 for an old pair that stays as an old-only (INACTIVE) pair: not a candidate, and with DROP not
// pristine either (status INACTIVE, p_n = k_pen = 0, z_t = 0)
template <bool DROP>
__global__ void k_merge_flags(xk_pairs old, const int32_t* __restrict__ cand, const int32_t* __restrict__ cstart,
                              long long nc, int32_t* __restrict__ r) {
  long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (o > old.n) return;
  if (o == old.n) { r[o] = 0; return; }
  const int a = old.ea[o], b = old.eb[o];
  long long l = lower_bound_cand(cand, cstart, a, b);
  bool found = l < nc && cand[2 * l] == a && cand[2 * l + 1] == b;
  bool stays = !found;
  if (DROP && stays) {
    const long long c = old.cap;
    stays = old.status[o] != 0 || old.p_n[o] != 0.0 || old.k_pen[o] != 0.0 || old.z_t[o] != 0.0 ||
            old.z_t[c + o] != 0.0;
  }
  r[o] = stays ? 1 : 0;
}

__global__ void k_merge_new(xk_pairs old, const int32_t* __restrict__ ostart, const int32_t* __restrict__ cand,
                            long long nc, const int32_t* __restrict__ R, xk_pairs out) {
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const int a = cand[2 * k], b = cand[2 * k + 1];
  long long lo = lower_bound_old(old, ostart, a, b);
  long long pos = k + R[lo];
  if (lo < old.n && old.ea[lo] == a && old.eb[lo] == b) {
    copy_state(old, lo, out, pos);
    return;
  }
  const long long cb = out.cap;
  out.ea[pos] = a;
  out.eb[pos] = b;
  out.s[pos] = 0.0;
  out.t[pos] = 0.0;
  out.gap[pos] = 0.0;
  for (int c = 0; c < 3; ++c) {
    out.normal[c * cb + pos] = 0.0;
    out.t1[c * cb + pos] = 0.0;
    out.t2[c * cb + pos] = 0.0;
  }
  out.lambda_n[pos] = 0.0;
  out.k_pen[pos] = 0.0;
  out.k_t[pos] = 0.0;
  out.p_n[pos] = 0.0;
  out.z_t[pos] = 0.0;
  out.z_t[cb + pos] = 0.0;
  out.q_trial_norm[pos] = 0.0;
  out.dissipation[pos] = 0.0;
  out.status[pos] = 0;
  out.stick[pos] = 1;
  if (out.coat_cc) {
    out.coat_cc[pos] = 0.0;
    out.coat_cc_prev[pos] = 0.0;
    out.coat_z_t[pos] = 0.0;
    out.coat_z_t[cb + pos] = 0.0;
    out.coat_qtn[pos] = 0.0;
    out.coat_diss[pos] = 0.0;
    out.coat_stick[pos] = 1;
  }
}

__global__ void k_merge_old(xk_pairs old, const int32_t* __restrict__ cand, const int32_t* __restrict__ cstart,
                            long long nc, const int32_t* __restrict__ r, const int32_t* __restrict__ R, xk_pairs out) {
  long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= old.n || !r[o]) return;
  long long pos = R[o] + lower_bound_cand(cand, cstart, old.ea[o], old.eb[o]);
  copy_state(old, o, out, pos);
  out.status[pos] = 0;  // INACTIVE
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

#define XK_TRY(x)                  \
  do {                             \
    xk_status r__ = (x);           \
    if (r__ != XK_OK) return r__;  \
  } while (0)

}  // namespace

// slot-list length of the walk: grows to the longest list seen (a power of two), kept for later calls
std::atomic<int> g_slot_cap{32};

extern "C" xk_status xk_broadphase(const xk_mesh* m, const double* u, const xk_bp_params* bp, int32_t* out_pairs,
                                   int64_t cap, int64_t* n_out, int64_t* n_raw, int64_t* n_prefilter, xk_stream s) {
  if (!m || !bp || !n_out) return xk_set_error(XK_ERR_ARG, "xk_broadphase: null argument");
  cudaStream_t st = (cudaStream_t)s;
  *n_out = 0;
  if (n_raw) *n_raw = 0;
  if (n_prefilter) *n_prefilter = 0;
  const long long ne = m->n_elems;
  if (ne < 2) return XK_OK;
  if (ne > 0x7fffffffLL) return xk_set_error(XK_ERR_OVERFLOW, "xk_broadphase: more than 2^31 segments");
  Scratch S{st};
  double* box;
  float4* boxf;
  double4_32a* mid;
  unsigned long long* ext;
  Grid* grid;
  XK_TRY(S.get(&box, 6 * ne));
  XK_TRY(S.get(&boxf, 2 * ne));
  XK_TRY(S.get(&mid, ne));
  XK_TRY(S.get(&ext, 16));
  XK_TRY(S.get(&grid, 1));
  // words: 0 unused, 1-3 lowest lower corner, 4-6 highest upper corner, 7 raw count, 8 the sum of the
  // box extents (a double, +0.0), 9-11 the largest extent on each axis, 12 the longest slot list
  double* ext_sum = reinterpret_cast<double*>(ext + 8);
  unsigned long long* raw_dev = ext + 7;
  int32_t* max_cnt = reinterpret_cast<int32_t*>(ext + 12);
  unsigned long long init[16] = {0ull, ~0ull, ~0ull, ~0ull, 0ull, 0ull, 0ull, 0ull,
                                 0ull, 0ull, 0ull, 0ull, 0ull, 0ull, 0ull, 0ull};
  XK_CUDA(cudaMemcpyAsync(ext, init, sizeof(init), cudaMemcpyHostToDevice, st));
  k_aabb<<<xk_blocks(ne, 256), 256, 0, st>>>(*m, u, bp->margin, box, boxf, mid, ext, ext_sum);
  // the grid has at most cap_cells cells, so the cell arrays are sized without reading it back
  const long long cap_cells = ne * 8 > 4096 ? ne * 8 : 4096;
  k_grid<<<1, 1, 0, st>>>(ext, ext_sum, ne, cap_cells, bp->cell_size, grid);
  XK_CHECK_LAUNCH();
  int32_t *segs, *cstart, *cfill, *cnt, *cnt2, *off2, *ecell;
  XK_TRY(S.get(&ecell, ne));
  XK_TRY(S.get(&segs, ne));
  XK_TRY(S.get(&cstart, cap_cells + 1));
  XK_TRY(S.get(&cfill, cap_cells + 1));
  XK_TRY(S.get(&cnt, ne + 1));
  XK_TRY(S.get(&cnt2, ne + 1));
  XK_TRY(S.get(&off2, ne + 1));
  // segments sorted by the cell of their lower corner
  XK_CUDA(cudaMemsetAsync(cfill, 0, sizeof(int32_t) * (cap_cells + 1), st));
  k_cell_count<<<xk_blocks(ne, 256), 256, 0, st>>>(box, ne, grid, ecell, cfill);
  XK_CHECK_LAUNCH();
  XK_TRY(xk_exclusive_scan_i32(cfill, cstart, cap_cells + 1, nullptr, st));
  XK_CUDA(cudaMemsetAsync(cfill, 0, sizeof(int32_t) * (cap_cells + 1), st));
  k_cell_scatter<<<xk_blocks(ne, 256), 256, 0, st>>>(ne, ecell, cstart, cfill, segs);
  k_cell_sort<<<xk_blocks(cap_cells, 256), 256, 0, st>>>(cap_cells, cstart, segs);
  XK_CHECK_LAUNCH();
  double *rsum, *part, *extra;
  int64_t* tot;
  XK_TRY(S.get(&rsum, ne));
  XK_TRY(S.get(&part, RED_BLOCKS));
  XK_TRY(S.get(&extra, 1));
  XK_TRY(S.get(&tot, 2));
  const int warp_blocks = xk_blocks(ne * 32, BP_T);
  const int excl_layer = (bp->exclude_same_layer && m->layer) ? 1 : 0;
  int slot_cap = g_slot_cap.load();
  for (int attempt = 0;; ++attempt) {
    if ((double)ne * slot_cap * 8.0 > 64.0e9)
      return xk_set_error(XK_ERR_OVERFLOW, "xk_broadphase: candidate lists too long for the slot buffers");
    int32_t *slot, *srt;
    XK_TRY(S.get(&slot, ne * slot_cap));
    XK_TRY(S.get(&srt, ne * slot_cap));
    XK_CUDA(cudaMemsetAsync(ext + 7, 0, sizeof(unsigned long long), st));
    XK_CUDA(cudaMemsetAsync(ext + 12, 0, sizeof(unsigned long long), st));
    k_sweep<<<warp_blocks, BP_T, 0, st>>>(*m, box, boxf, grid, segs, cstart, bp->exclude_shared, excl_layer,
                                          slot_cap, slot, cnt, rsum, raw_dev, max_cnt);
    XK_CHECK_LAUNCH();
    XK_TRY(xk_exclusive_scan_i32(cnt, off2, ne, tot, st));  // tot[0]: candidates before the prescreen
    const double* ex = nullptr;
    if (bp->midpoint_prescreening) {
      if (!(bp->prescreening_margin > 0.0)) k_radsum_partial<<<RED_BLOCKS, RED_T, 0, st>>>(rsum, ne, part);
      k_margin<<<1, 1, 0, st>>>(part, tot, bp->prescreening_margin, extra);
      XK_CHECK_LAUNCH();
      ex = extra;
    }
    k_slots_rank<<<warp_blocks, BP_T, 0, st>>>(*m, mid, slot, cnt, slot_cap, ex, srt, cnt2);
    XK_CHECK_LAUNCH();
    XK_TRY(xk_exclusive_scan_i32(cnt2, off2, ne, tot + 1, st));
    k_slots_emit<<<warp_blocks, BP_T, 0, st>>>(ne, srt, cnt, slot_cap, off2, cap, out_pairs);
    XK_CHECK_LAUNCH();
    int64_t h[2];
    unsigned long long hw[2] = {0ull, 0ull};
    XK_CUDA(cudaMemcpyAsync(h, tot, sizeof(h), cudaMemcpyDeviceToHost, st));
    XK_CUDA(cudaMemcpyAsync(hw, ext + 7, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    XK_CUDA(cudaMemcpyAsync(hw + 1, ext + 12, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    XK_CUDA(cudaStreamSynchronize(st));
    const int longest = (int)(uint32_t)hw[1];
    if (longest > slot_cap) {  // some lists were cut short: walk again with lists long enough for all
      if (attempt > 0) return xk_set_error(XK_ERR_OVERFLOW, "xk_broadphase: slot lists overflowed twice");
      int c = slot_cap;
      while (c < longest) c *= 2;
      slot_cap = c;
      int prev = g_slot_cap.load();
      while (prev < c && !g_slot_cap.compare_exchange_weak(prev, c)) {
      }
      continue;
    }
    if (h[1] > 0x7fffffffLL) return xk_set_error(XK_ERR_OVERFLOW, "xk_broadphase: more than 2^31 candidates");
    if (n_raw) *n_raw = (int64_t)hw[0];
    if (n_prefilter) *n_prefilter = h[0];
    *n_out = h[1];
    if (h[1] > cap) return xk_set_error(XK_ERR_CAPACITY, "xk_broadphase: output capacity too small");
    return XK_OK;
  }
}

static xk_status merge_impl(const xk_mesh* m, const xk_pairs* old, const int32_t* cands, int64_t n_cands,
                            xk_pairs* out, xk_stream s, bool drop) {
  if (!m || !old || !out || (n_cands > 0 && !cands)) return xk_set_error(XK_ERR_ARG, "xk_pairs_merge: null argument");
  if ((long long)out->cap < (long long)old->n + n_cands)
    return xk_set_error(XK_ERR_CAPACITY, "xk_pairs_merge: out->cap < old->n + n_cands");
  cudaStream_t st = (cudaStream_t)s;
  Scratch S{st};
  int32_t *r, *R, *ostart, *cstart;
  int64_t* tot;
  const long long ne = m->n_elems;
  XK_TRY(S.get(&r, (long long)old->n + 1));
  XK_TRY(S.get(&R, (long long)old->n + 1));
  XK_TRY(S.get(&ostart, ne + 2));
  XK_TRY(S.get(&cstart, ne + 2));
  XK_TRY(S.get(&tot, 1));
  // per-segment row ranges of both sorted lists: each lookup searches only its segment's rows
  k_seg_start<1><<<xk_blocks(ne + 1, 256), 256, 0, st>>>(old->ea, old->n, ne, ostart);
  k_seg_start<2><<<xk_blocks(ne + 1, 256), 256, 0, st>>>(cands, n_cands, ne, cstart);
  if (drop)
    k_merge_flags<true><<<xk_blocks((long long)old->n + 1, 256), 256, 0, st>>>(*old, cands, cstart, n_cands, r);
  else
    k_merge_flags<false><<<xk_blocks((long long)old->n + 1, 256), 256, 0, st>>>(*old, cands, cstart, n_cands, r);
  XK_CHECK_LAUNCH();
  XK_TRY(xk_exclusive_scan_i32(r, R, (long long)old->n + 1, tot, st));
  if (n_cands > 0) k_merge_new<<<xk_blocks(n_cands, 256), 256, 0, st>>>(*old, ostart, cands, n_cands, R, *out);
  if (old->n > 0) k_merge_old<<<xk_blocks(old->n, 256), 256, 0, st>>>(*old, cands, cstart, n_cands, r, R, *out);
  XK_CHECK_LAUNCH();
  int64_t h = 0;
  XK_CUDA(cudaMemcpyAsync(&h, tot, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  XK_CUDA(cudaStreamSynchronize(st));
  out->n = (int32_t)(n_cands + h);
  return XK_OK;
}

extern "C" xk_status xk_pairs_merge(const xk_mesh* m, const xk_pairs* old, const int32_t* cands, int64_t n_cands,
                                    xk_pairs* out, xk_stream s) {
  return merge_impl(m, old, cands, n_cands, out, s, false);
}

extern "C" xk_status xk_pairs_merge_pruned(const xk_mesh* m, const xk_pairs* old, const int32_t* cands,
                                           int64_t n_cands, xk_pairs* out, xk_stream s) {
  return merge_impl(m, old, cands, n_cands, out, s, true);
}
