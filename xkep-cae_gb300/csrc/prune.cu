// Learned pruning of broadphase candidate pairs: per-candidate features, a
// small MLP (F = 8 inputs -> 64 -> 64 -> 64 -> 1, ReLU, BF16 weights and
// activations, FP32 accumulation), its training kernels (forward with stored
// activations, backward, deterministic weight-gradient reduction, Adam) and the
// selection / pair-table compaction that apply it at detection time.
//
// Inference runs on the tensor cores (mma.sync m16n8k16 BF16 -> FP32): a warp
// takes 16 candidates, and each layer's accumulator fragments are rounded to
// BF16 and re-packed in registers as the next layer's A operand.  Training runs
// one sample per thread in FP32 on BF16-rounded operands, which is the same
// arithmetic up to the order of the float sums.
#include <cuda_bf16.h>

#include "xk_common.cuh"

namespace {

constexpr int MF = XK_MLP_IN, MH = XK_MLP_HIDDEN, NP = XK_MLP_PARAMS, NA = XK_MLP_ACT;
constexpr int O_W1 = 0, O_B1 = O_W1 + MH * MF, O_W2 = O_B1 + MH, O_B2 = O_W2 + MH * MH, O_W3 = O_B2 + MH,
              O_B3 = O_W3 + MH * MH, O_W4 = O_B3 + MH, O_B4 = O_W4 + MH;
static_assert(O_B4 + 1 == NP, "parameter layout");
static_assert(NA == 3 * MH, "activation layout");

XK_D float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

XK_D uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x (low half) = lo
  return *reinterpret_cast<uint32_t*>(&v);
}

XK_D float bf16_at(const uint16_t* w, int i) {
  return __uint_as_float(((uint32_t)w[i]) << 16);
}

// D = A * B + D for one m16n8k16 tile (A row-major 16x16, B "col" 16x8, BF16 in, FP32 accumulate).
XK_D void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ------------------------------------------------------------------ features

// Exact double arithmetic in the order of the oracle's NumPy expressions, cast to float at the end.
__global__ void k_features(xk_mesh m, const double* __restrict__ u, const int32_t* __restrict__ cands, long long n,
                           xk_pairs old, float* __restrict__ feat, uint8_t* __restrict__ hist) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ea = cands[2 * i], eb = cands[2 * i + 1];
  const int nd[4] = {m.conn[2 * ea], m.conn[2 * ea + 1], m.conn[2 * eb], m.conn[2 * eb + 1]};
  double x[4][3];
  for (int k = 0; k < 4; ++k)
    for (int c = 0; c < 3; ++c)
      x[k][c] = u ? xadd(m.X[3LL * nd[k] + c], u[6LL * nd[k] + c]) : m.X[3LL * nd[k] + c];
  const double rs = xadd(m.radii[ea], m.radii[eb]);
  double dm[3], da[3], db[3];
  for (int c = 0; c < 3; ++c) {
    const double ma = xmul(0.5, xadd(x[0][c], x[1][c])), mb = xmul(0.5, xadd(x[2][c], x[3][c]));
    dm[c] = xsub(ma, mb);
    da[c] = xsub(x[1][c], x[0][c]);
    db[c] = xsub(x[3][c], x[2][c]);
  }
  const double sep = xsqrt(xdot_seq(dm, dm));
  const double lna = xsqrt(xdot_seq(da, da)), lnb = xsqrt(xdot_seq(db, db));
  double den = xmul(lna, lnb);
  if (!(den >= 1e-300)) den = (den != den) ? den : 1e-300;
  const double cosv = xdiv(fabs(xdot_seq(da, db)), den);
  float f[MF];
  f[0] = (float)xdiv(sep, rs);
  f[1] = (float)cosv;
  f[2] = (float)xdiv(xadd(lna, lnb), xmul(2.0, rs));
  const int la = m.layer ? m.layer[ea] : -1, lb = m.layer ? m.layer[eb] : -1;
  const bool have = la >= 0 && lb >= 0;
  const int dl = la > lb ? la - lb : lb - la;
  f[3] = have ? (float)xdiv((double)(dl < 3 ? dl : 3), 3.0) : 0.f;
  f[4] = (have && (la == 0 || lb == 0)) ? 1.f : 0.f;
  // previous-step gap: the pair in the old table (sorted by (ea, eb))
  long long lo = 0, hi = (long long)old.n - 1, at = -1;
  while (lo <= hi) {
    const long long mid = (lo + hi) >> 1;
    const int oa = old.ea[mid], ob = old.eb[mid];
    if (oa == ea && ob == eb) { at = mid; break; }
    if (oa < ea || (oa == ea && ob < eb)) lo = mid + 1; else hi = mid - 1;
  }
  double g5;
  if (at >= 0) {
    g5 = xdiv(old.gap[at], rs);
  } else {
    g5 = xdiv(xsub(xsub(sep, xmul(0.5, xadd(lna, lnb))), rs), rs);
  }
  g5 = g5 < -2.0 ? -2.0 : (g5 > 8.0 ? 8.0 : g5);
  f[5] = (float)g5;
  f[6] = at >= 0 ? 1.f : 0.f;
  f[7] = 0.f;
  float4* o = reinterpret_cast<float4*>(feat + MF * i);
  o[0] = make_float4(f[0], f[1], f[2], f[3]);
  o[1] = make_float4(f[4], f[5], f[6], f[7]);
  uint8_t h = 0;
  if (at >= 0) {
    const long long c = old.cap;
    h = (old.status[at] != 0 || old.p_n[at] > 0.0 || old.k_pen[at] > 0.0 || old.z_t[at] != 0.0 ||
         old.z_t[c + at] != 0.0) ? 1 : 0;
  }
  hist[i] = h;
}

// ------------------------------------------------------------------ inference (tensor cores)

constexpr int FW_WARPS = 4;

__global__ void __launch_bounds__(32 * FW_WARPS) k_mlp_forward_mma(const uint16_t* __restrict__ P,
                                                                   const float* __restrict__ feat, long long n,
                                                                   float* __restrict__ logit) {
  __shared__ __align__(16) uint16_t W[NP + 7];
  for (int i = threadIdx.x; i < NP; i += blockDim.x) W[i] = P[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const long long tiles = (n + 15) / 16;
  const uint32_t* W32 = reinterpret_cast<const uint32_t*>(W);
  for (long long tile = (long long)blockIdx.x * FW_WARPS + (threadIdx.x >> 5); tile < tiles;
       tile += (long long)gridDim.x * FW_WARPS) {
    const long long r0 = tile * 16 + g, r1 = r0 + 8;
    uint32_t a[4][4];
    {
      float2 x0 = r0 < n ? *reinterpret_cast<const float2*>(feat + MF * r0 + 2 * t) : make_float2(0.f, 0.f);
      float2 x1 = r1 < n ? *reinterpret_cast<const float2*>(feat + MF * r1 + 2 * t) : make_float2(0.f, 0.f);
      a[0][0] = pack_bf16(x0.x, x0.y);
      a[0][1] = pack_bf16(x1.x, x1.y);
      a[0][2] = 0u;  // k = 8..15: no inputs
      a[0][3] = 0u;
    }
    float c[8][4];
    // layer 1: K = 16 (8 inputs + zero padding)
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int j = nt * 8 + 2 * t;
      c[nt][0] = c[nt][2] = bf16_at(W, O_B1 + j);
      c[nt][1] = c[nt][3] = bf16_at(W, O_B1 + j + 1);
      mma_bf16(c[nt], a[0], W32[(O_W1 + (nt * 8 + g) * MF + 2 * t) >> 1], 0u);
    }
    // layers 2 and 3: K = 64 as 4 k-tiles; the relu'd, rounded accumulators are the next A operand
#pragma unroll
    for (int layer = 0; layer < 2; ++layer) {
      const int ow = layer == 0 ? O_W2 : O_W3, ob = layer == 0 ? O_B2 : O_B3;
#pragma unroll
      for (int kt = 0; kt < 4; ++kt) {
        a[kt][0] = pack_bf16(fmaxf(c[2 * kt][0], 0.f), fmaxf(c[2 * kt][1], 0.f));
        a[kt][1] = pack_bf16(fmaxf(c[2 * kt][2], 0.f), fmaxf(c[2 * kt][3], 0.f));
        a[kt][2] = pack_bf16(fmaxf(c[2 * kt + 1][0], 0.f), fmaxf(c[2 * kt + 1][1], 0.f));
        a[kt][3] = pack_bf16(fmaxf(c[2 * kt + 1][2], 0.f), fmaxf(c[2 * kt + 1][3], 0.f));
      }
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        const int j = nt * 8 + 2 * t;
        c[nt][0] = c[nt][2] = bf16_at(W, ob + j);
        c[nt][1] = c[nt][3] = bf16_at(W, ob + j + 1);
        const int row = ow + (nt * 8 + g) * MH;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
          mma_bf16(c[nt], a[kt], W32[(row + kt * 16 + 2 * t) >> 1], W32[(row + kt * 16 + 8 + 2 * t) >> 1]);
      }
    }
    // output: logit = b4 + sum_k bf16(relu(z3_k)) w4_k, the row sum over the quad
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int j = nt * 8 + 2 * t;
      const float w0 = bf16_at(W, O_W4 + j), w1 = bf16_at(W, O_W4 + j + 1);
      s0 += bf16r(fmaxf(c[nt][0], 0.f)) * w0 + bf16r(fmaxf(c[nt][1], 0.f)) * w1;
      s1 += bf16r(fmaxf(c[nt][2], 0.f)) * w0 + bf16r(fmaxf(c[nt][3], 0.f)) * w1;
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    if (t == 0) {
      const float b4 = bf16_at(W, O_B4);
      if (r0 < n) logit[r0] = s0 + b4;
      if (r1 < n) logit[r1] = s1 + b4;
    }
  }
}

// ------------------------------------------------------------------ training (one sample per thread)

constexpr int TR_T = 128;

// Activations and deltas are stored plane-major: value q of sample i at [q * n + i].
// The outer loops over units run at run time and the 64-wide dot products are
// unrolled; a layer's input vector is read back from its (just written) plane
// into registers, so no register array is indexed at run time.
__global__ void __launch_bounds__(TR_T) k_mlp_train_fwd(const float* __restrict__ theta,
                                                        const float* __restrict__ feat, long long n,
                                                        float* __restrict__ act, float* __restrict__ logit) {
  __shared__ float W[NP];
  for (int i = threadIdx.x; i < NP; i += blockDim.x) W[i] = bf16r(theta[i]);
  __syncthreads();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x[MF];
#pragma unroll
  for (int k = 0; k < MF; ++k) x[k] = bf16r(feat[MF * i + k]);
#pragma unroll 1
  for (int j = 0; j < MH; ++j) {
    float z = 0.f;
#pragma unroll
    for (int k = 0; k < MF; ++k) z += W[O_W1 + j * MF + k] * x[k];
    act[(long long)j * n + i] = bf16r(fmaxf(z + W[O_B1 + j], 0.f));
  }
  float a[MH];
#pragma unroll 1
  for (int layer = 0; layer < 2; ++layer) {
    const int ow = layer == 0 ? O_W2 : O_W3, ob = layer == 0 ? O_B2 : O_B3;
#pragma unroll
    for (int k = 0; k < MH; ++k) a[k] = act[(long long)(layer * MH + k) * n + i];
#pragma unroll 1
    for (int j = 0; j < MH; ++j) {
      float z = 0.f;
#pragma unroll
      for (int k = 0; k < MH; ++k) z += W[ow + j * MH + k] * a[k];
      act[(long long)((layer + 1) * MH + j) * n + i] = bf16r(fmaxf(z + W[ob + j], 0.f));
    }
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < MH; ++k) s += act[(long long)(2 * MH + k) * n + i] * W[O_W4 + k];
  logit[i] = s + W[O_B4];
}

__global__ void __launch_bounds__(TR_T) k_mlp_train_bwd(const float* __restrict__ theta, const float* __restrict__ act,
                                                        const float* __restrict__ logit, const float* __restrict__ y,
                                                        const float* __restrict__ w, long long n,
                                                        float* __restrict__ dvec, float* __restrict__ gout,
                                                        double* __restrict__ loss_part) {
  __shared__ float W[NP];
  __shared__ double red[TR_T];
  for (int i = threadIdx.x; i < NP; i += blockDim.x) W[i] = bf16r(theta[i]);
  __syncthreads();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double li = 0.0;
  if (i < n) {
    const double l = (double)logit[i], yi = (double)y[i], wi = (double)w[i];
    const double sp = l > 0.0 ? l + log1p(exp(-l)) : log1p(exp(l));
    li = wi * (sp - yi * l) / (double)n;
    const float g = (float)(wi * (1.0 / (1.0 + exp(-l)) - yi) / (double)n);
    gout[i] = g;
#pragma unroll 1
    for (int k = 0; k < MH; ++k)
      dvec[(long long)(2 * MH + k) * n + i] = act[(long long)(2 * MH + k) * n + i] > 0.f ? g * W[O_W4 + k] : 0.f;
    // d2 = (W3^T d3) masked, then d1 = (W2^T d2) masked
    float d[MH];
#pragma unroll 1
    for (int layer = 1; layer >= 0; --layer) {
      const int ow = layer == 1 ? O_W3 : O_W2;
#pragma unroll
      for (int j = 0; j < MH; ++j) d[j] = dvec[(long long)((layer + 1) * MH + j) * n + i];
#pragma unroll 1
      for (int k = 0; k < MH; ++k) {
        float z = 0.f;
#pragma unroll
        for (int j = 0; j < MH; ++j) z += W[ow + j * MH + k] * d[j];
        const long long q = (long long)(layer * MH + k) * n + i;
        dvec[q] = act[q] > 0.f ? z : 0.f;
      }
    }
  }
  red[threadIdx.x] = li;
  __syncthreads();
  for (int s = TR_T / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0];
}

// Weight gradients: each block sums its chunk of samples for every parameter
// (fixed order); a second kernel adds the block partials in block order.
constexpr int WG_T = 256, WG_CHUNK = 1024, WG_SUB = 16, WG_SLOTS = (NP + WG_T - 1) / WG_T;

__global__ void __launch_bounds__(WG_T) k_mlp_wgrad(const float* __restrict__ feat, const float* __restrict__ act,
                                                    const float* __restrict__ dvec, const float* __restrict__ g,
                                                    long long n, float* __restrict__ partial) {
  __shared__ float Ds[WG_SUB][NA + 1];      // d1 d2 d3 | g
  __shared__ float As[WG_SUB][MF + NA + 1];  // x0 a1 a2 a3 | 1
  int drow[WG_SLOTS], acol[WG_SLOTS];
  float acc[WG_SLOTS];
#pragma unroll
  for (int q = 0; q < WG_SLOTS; ++q) {
    const int p = threadIdx.x + WG_T * q;
    int dr = 0, ac = MF + NA;
    if (p < O_B1) { dr = (p - O_W1) / MF; ac = (p - O_W1) % MF; }
    else if (p < O_W2) { dr = p - O_B1; }
    else if (p < O_B2) { dr = MH + (p - O_W2) / MH; ac = MF + (p - O_W2) % MH; }
    else if (p < O_W3) { dr = MH + (p - O_B2); }
    else if (p < O_B3) { dr = 2 * MH + (p - O_W3) / MH; ac = MF + MH + (p - O_W3) % MH; }
    else if (p < O_W4) { dr = 2 * MH + (p - O_B3); }
    else if (p < O_B4) { dr = NA; ac = MF + 2 * MH + (p - O_W4); }
    else { dr = NA; }
    drow[q] = dr;
    acol[q] = ac;
    acc[q] = 0.f;
  }
  const long long c0 = (long long)blockIdx.x * WG_CHUNK;
  const long long c1 = (c0 + WG_CHUNK < n) ? c0 + WG_CHUNK : n;
  for (long long s0 = c0; s0 < c1; s0 += WG_SUB) {
    const int ns = (int)((c1 - s0) < WG_SUB ? (c1 - s0) : WG_SUB);
    for (int e = threadIdx.x; e < WG_SUB * (NA + 1); e += WG_T) {
      const int s = e % WG_SUB, q = e / WG_SUB;
      float v = 0.f;
      if (s < ns) v = q < NA ? dvec[(long long)q * n + s0 + s] : g[s0 + s];
      Ds[s][q] = v;
    }
    for (int e = threadIdx.x; e < WG_SUB * (MF + NA + 1); e += WG_T) {
      const int s = e % WG_SUB, q = e / WG_SUB;
      float v = 0.f;
      if (s < ns) {
        if (q < MF) v = bf16r(feat[MF * (s0 + s) + q]);
        else if (q < MF + NA) v = act[(long long)(q - MF) * n + s0 + s];
        else v = 1.f;
      }
      As[s][q] = v;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < WG_SLOTS; ++q) {
      if (threadIdx.x + WG_T * q < NP) {
        float a = acc[q];
#pragma unroll
        for (int s = 0; s < WG_SUB; ++s) a += Ds[s][drow[q]] * As[s][acol[q]];
        acc[q] = a;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < WG_SLOTS; ++q) {
    const int p = threadIdx.x + WG_T * q;
    if (p < NP) partial[(long long)blockIdx.x * NP + p] = acc[q];
  }
}

__global__ void k_sum_partials(const float* __restrict__ partial, int nb, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NP) return;
  float s = 0.f;
  for (int b = 0; b < nb; ++b) s += partial[(long long)b * NP + p];
  grad[p] = s;
}

__global__ void k_sum_loss(const double* __restrict__ part, int nb, float* __restrict__ loss) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += part[b];
    *loss = (float)s;
  }
}

// Adam with the float32 roundings of the oracle's NumPy expressions (no contraction).
__global__ void k_adam(float* __restrict__ theta, const float* __restrict__ grad, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float ob1, float b2, float ob2, float bc1, float bc2,
                       float eps, uint16_t* __restrict__ out_bf16) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NP) return;
  const float gr = grad[p];
  const float mm = __fadd_rn(__fmul_rn(b1, m[p]), __fmul_rn(ob1, gr));
  const float vv = __fadd_rn(__fmul_rn(b2, v[p]), __fmul_rn(__fmul_rn(ob2, gr), gr));
  const float mh = __fdiv_rn(mm, bc1), vh = __fdiv_rn(vv, bc2);
  const float th = __fsub_rn(theta[p], __fdiv_rn(__fmul_rn(lr, mh), __fadd_rn(__fsqrt_rn(vh), eps)));
  m[p] = mm;
  v[p] = vv;
  theta[p] = th;
  if (out_bf16) {
    __nv_bfloat16 h = __float2bfloat16_rn(th);
    out_bf16[p] = *reinterpret_cast<uint16_t*>(&h);
  }
}

__global__ void k_to_bf16(const float* __restrict__ theta, uint16_t* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NP) return;
  __nv_bfloat16 h = __float2bfloat16_rn(theta[p]);
  out[p] = *reinterpret_cast<uint16_t*>(&h);
}

// ------------------------------------------------------------------ selection and table compaction

__global__ void k_keep_flags(long long n, const float* __restrict__ logit, const uint8_t* __restrict__ hist,
                             float thr, int invert, int32_t* __restrict__ flag) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const int keep = (logit[i] >= thr || (hist && hist[i])) ? 1 : 0;
    flag[i] = invert ? 1 - keep : keep;
  }
}

__global__ void k_scatter_cands(long long n, const int32_t* __restrict__ cands, const int32_t* __restrict__ flag,
                                const int32_t* __restrict__ off, int32_t* __restrict__ kept) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) {
    const long long o = off[i];
    kept[2 * o] = cands[2 * i];
    kept[2 * o + 1] = cands[2 * i + 1];
  }
}

__global__ void k_old_keep(xk_pairs p, const int32_t* __restrict__ kept, long long nk, int32_t* __restrict__ flag) {
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.n) return;
  const long long c = p.cap;
  const bool pristine = p.status[j] == 0 && p.p_n[j] == 0.0 && p.k_pen[j] == 0.0 && p.z_t[j] == 0.0 &&
                        p.z_t[c + j] == 0.0;
  int keep = 1;
  if (pristine) {
    const int ea = p.ea[j], eb = p.eb[j];
    long long lo = 0, hi = nk - 1;
    keep = 0;
    while (lo <= hi) {
      const long long mid = (lo + hi) >> 1;
      const int a = kept[2 * mid], b = kept[2 * mid + 1];
      if (a == ea && b == eb) { keep = 1; break; }
      if (a < ea || (a == ea && b < eb)) lo = mid + 1; else hi = mid - 1;
    }
  }
  flag[j] = keep;
}

__global__ void k_compact_table(xk_pairs in, const int32_t* __restrict__ flag, const int32_t* __restrict__ off,
                                xk_pairs out) {
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= in.n || !flag[j]) return;
  const long long o = off[j], ci = in.cap, co = out.cap;
  out.ea[o] = in.ea[j];
  out.eb[o] = in.eb[j];
  out.s[o] = in.s[j];
  out.t[o] = in.t[j];
  out.gap[o] = in.gap[j];
  for (int c = 0; c < 3; ++c) {
    out.normal[c * co + o] = in.normal[c * ci + j];
    out.t1[c * co + o] = in.t1[c * ci + j];
    out.t2[c * co + o] = in.t2[c * ci + j];
  }
  out.lambda_n[o] = in.lambda_n[j];
  out.k_pen[o] = in.k_pen[j];
  out.k_t[o] = in.k_t[j];
  out.p_n[o] = in.p_n[j];
  out.z_t[o] = in.z_t[j];
  out.z_t[co + o] = in.z_t[ci + j];
  out.q_trial_norm[o] = in.q_trial_norm[j];
  out.dissipation[o] = in.dissipation[j];
  out.status[o] = in.status[j];
  out.stick[o] = in.stick[j];
}

}  // namespace

// ------------------------------------------------------------------ entry points

extern "C" xk_status xk_prune_features(const xk_mesh* m, const double* u, const int32_t* cands, int64_t n,
                                       const xk_pairs* old, float* feat, uint8_t* hist, xk_stream s) {
  if (!m || !old || (n > 0 && (!cands || !feat || !hist)) || n < 0)
    return xk_set_error(XK_ERR_ARG, "xk_prune_features: bad arguments");
  if (n == 0) return XK_OK;
  k_features<<<xk_blocks(n, 256), 256, 0, (cudaStream_t)s>>>(*m, u, cands, n, *old, feat, hist);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_mlp_forward(const uint16_t* params_bf16, const float* feat, int64_t n, float* logit,
                                    xk_stream s) {
  if (!params_bf16 || n < 0 || (n > 0 && (!feat || !logit)))
    return xk_set_error(XK_ERR_ARG, "xk_mlp_forward: bad arguments");
  if (n == 0) return XK_OK;
  const long long tiles = (n + 15) / 16;
  long long blocks = (tiles + FW_WARPS - 1) / FW_WARPS;
  if (blocks > 152 * 16) blocks = 152 * 16;  // grid-stride beyond 16 blocks per SM
  k_mlp_forward_mma<<<(int)blocks, 32 * FW_WARPS, 0, (cudaStream_t)s>>>(params_bf16, feat, n, logit);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_mlp_train_forward(const float* theta, const float* feat, int64_t n, float* act,
                                          float* logit, xk_stream s) {
  if (!theta || n < 0 || (n > 0 && (!feat || !act || !logit)))
    return xk_set_error(XK_ERR_ARG, "xk_mlp_train_forward: bad arguments");
  if (n == 0) return XK_OK;
  k_mlp_train_fwd<<<xk_blocks(n, TR_T), TR_T, 0, (cudaStream_t)s>>>(theta, feat, n, act, logit);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_mlp_backward(const float* theta, const float* feat, const float* act, const float* logit,
                                     const float* y, const float* w, int64_t n, float* dvec, float* g, float* grad,
                                     float* loss, xk_stream s) {
  if (!theta || !grad || !loss || n <= 0 || !feat || !act || !logit || !y || !w || !dvec || !g)
    return xk_set_error(XK_ERR_ARG, "xk_mlp_backward: bad arguments");
  cudaStream_t st = (cudaStream_t)s;
  const int nb_t = xk_blocks(n, TR_T);
  const int nb_w = (int)((n + WG_CHUNK - 1) / WG_CHUNK);
  double* lpart = nullptr;
  float* part = nullptr;
  XK_CUDA(cudaMallocAsync((void**)&lpart, sizeof(double) * nb_t, st));
  cudaError_t e = cudaMallocAsync((void**)&part, sizeof(float) * (size_t)nb_w * NP, st);
  if (e != cudaSuccess) {
    cudaFreeAsync(lpart, st);
    return xk_set_cuda_error(e, __FILE__, __LINE__);
  }
  k_mlp_train_bwd<<<nb_t, TR_T, 0, st>>>(theta, act, logit, y, w, n, dvec, g, lpart);
  k_sum_loss<<<1, 32, 0, st>>>(lpart, nb_t, loss);
  k_mlp_wgrad<<<nb_w, WG_T, 0, st>>>(feat, act, dvec, g, n, part);
  k_sum_partials<<<(NP + 255) / 256, 256, 0, st>>>(part, nb_w, grad);
  e = cudaGetLastError();
  cudaFreeAsync(lpart, st);
  cudaFreeAsync(part, st);
  if (e != cudaSuccess) return xk_set_cuda_error(e, __FILE__, __LINE__);
  return XK_OK;
}

extern "C" xk_status xk_mlp_adam(float* theta, const float* grad, float* m, float* v, int step, double lr,
                                 double beta1, double beta2, double eps, uint16_t* theta_bf16, xk_stream s) {
  if (!theta || !grad || !m || !v || step < 1) return xk_set_error(XK_ERR_ARG, "xk_mlp_adam: bad arguments");
  // each constant is formed in double and rounded to float once
  const float ob1 = (float)(1.0 - beta1), ob2 = (float)(1.0 - beta2);
  const float bc1 = (float)(1.0 - pow(beta1, step)), bc2 = (float)(1.0 - pow(beta2, step));
  k_adam<<<(NP + 255) / 256, 256, 0, (cudaStream_t)s>>>(theta, grad, m, v, (float)lr, (float)beta1, ob1,
                                                        (float)beta2, ob2, bc1, bc2, (float)eps, theta_bf16);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_mlp_to_bf16(const float* theta, uint16_t* out, xk_stream s) {
  if (!theta || !out) return xk_set_error(XK_ERR_ARG, "xk_mlp_to_bf16: bad arguments");
  k_to_bf16<<<(NP + 255) / 256, 256, 0, (cudaStream_t)s>>>(theta, out);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_prune_select(const int32_t* cands, int64_t n, const float* logit, const uint8_t* hist,
                                     float threshold, int invert, int32_t* kept, int64_t* n_kept, xk_stream s) {
  if (!n_kept || n < 0 || (n > 0 && (!cands || !logit || !kept)))
    return xk_set_error(XK_ERR_ARG, "xk_prune_select: bad arguments");
  *n_kept = 0;
  if (n == 0) return XK_OK;
  cudaStream_t st = (cudaStream_t)s;
  int32_t* flag = nullptr;
  int64_t* tot = nullptr;
  XK_CUDA(cudaMallocAsync((void**)&flag, sizeof(int32_t) * 2 * n, st));
  cudaError_t e = cudaMallocAsync((void**)&tot, sizeof(int64_t), st);
  if (e != cudaSuccess) {
    cudaFreeAsync(flag, st);
    return xk_set_cuda_error(e, __FILE__, __LINE__);
  }
  int32_t* off = flag + n;
  k_keep_flags<<<xk_blocks(n, 256), 256, 0, st>>>(n, logit, hist, threshold, invert, flag);
  xk_status r = xk_exclusive_scan_i32(flag, off, n, tot, st);
  if (r == XK_OK) {
    k_scatter_cands<<<xk_blocks(n, 256), 256, 0, st>>>(n, cands, flag, off, kept);
    int64_t h = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, tot, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) r = xk_set_cuda_error(e, __FILE__, __LINE__);
    else *n_kept = h;
  }
  cudaFreeAsync(flag, st);
  cudaFreeAsync(tot, st);
  return r;
}

extern "C" xk_status xk_pairs_drop_pristine(const xk_pairs* in, const int32_t* kept, int64_t n_kept, xk_pairs* out,
                                            xk_stream s) {
  if (!in || !out || n_kept < 0 || (n_kept > 0 && !kept))
    return xk_set_error(XK_ERR_ARG, "xk_pairs_drop_pristine: bad arguments");
  cudaStream_t st = (cudaStream_t)s;
  out->n = 0;
  if (in->n == 0) return XK_OK;
  int32_t* flag = nullptr;
  int64_t* tot = nullptr;
  const long long n = in->n;
  XK_CUDA(cudaMallocAsync((void**)&flag, sizeof(int32_t) * 2 * n, st));
  cudaError_t e = cudaMallocAsync((void**)&tot, sizeof(int64_t), st);
  if (e != cudaSuccess) {
    cudaFreeAsync(flag, st);
    return xk_set_cuda_error(e, __FILE__, __LINE__);
  }
  int32_t* off = flag + n;
  k_old_keep<<<xk_blocks(n, 256), 256, 0, st>>>(*in, kept, n_kept, flag);
  xk_status r = xk_exclusive_scan_i32(flag, off, n, tot, st);
  int64_t h = 0;
  if (r == XK_OK) {
    e = cudaMemcpyAsync(&h, tot, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) r = xk_set_cuda_error(e, __FILE__, __LINE__);
  }
  if (r == XK_OK && h > out->cap) r = xk_set_error(XK_ERR_CAPACITY, "xk_pairs_drop_pristine: out->cap too small");
  if (r == XK_OK) {
    k_compact_table<<<xk_blocks(n, 256), 256, 0, st>>>(*in, flag, off, *out);
    e = cudaGetLastError();
    if (e != cudaSuccess) r = xk_set_cuda_error(e, __FILE__, __LINE__);
    else out->n = (int32_t)h;
  }
  cudaFreeAsync(flag, st);
  cudaFreeAsync(tot, st);
  return r;
}
