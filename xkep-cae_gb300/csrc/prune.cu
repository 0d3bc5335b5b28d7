// Learned pruning of broadphase candidate pairs: per-candidate features, a
// small MLP (F = 8 inputs -> 64 -> 64 -> 64 -> 1, ReLU, BF16 weights and
// activations, FP32 accumulation), its training kernels (forward with stored
// activations, backward, deterministic weight-gradient reduction, Adam) and the
// selection / pair-table compaction that apply it at detection time.
//
// Inference runs on the tensor cores, in two forms: tcgen05.mma with the
// accumulator in TMEM, 128 candidates per CTA tile (the default), and
// mma.sync m16n8k16 (BF16 -> FP32), where a warp takes 16 candidates and each
// layer's accumulator fragments are re-packed in registers as the next layer's
// A operand.  Training runs
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

// Current gap of a candidate over (r_a + r_b), in float, from the segment differences a3 = a1 - a0,
// b3 = b1 - b0, w3 = a0 - b0: the clamped closest-point parameters of _closest_point_segments_batch
// (geometry/_compute.py:55-151) in float, each product and sum rounded on its own (no contraction),
// so that a NumPy float32 restatement gives the same value; near-parallel pairs (det <= 1e-3 ac)
// take s = 0.
XK_D float current_gap_f(const float* a3, const float* b3, const float* w3, float rsf) {
  auto dotf = [](const float* p, const float* q) {
    return __fadd_rn(__fadd_rn(__fmul_rn(p[0], q[0]), __fmul_rn(p[1], q[1])), __fmul_rn(p[2], q[2]));
  };
  auto clampf = [](float v) { return v < 0.f ? 0.f : (v > 1.f ? 1.f : v); };
  const float a = dotf(a3, a3), b = dotf(a3, b3), c = dotf(b3, b3), d = dotf(a3, w3), e = dotf(b3, w3);
  const float ac = __fmul_rn(a, c);
  const float det = __fsub_rn(ac, __fmul_rn(b, b));
  float s, t;
  if (!(det > __fmul_rn(1e-3f, ac))) {
    s = 0.f;
    t = c > 0.f ? clampf(__fdiv_rn(e, c)) : 0.f;
  } else {
    const float su = __fdiv_rn(__fsub_rn(__fmul_rn(b, e), __fmul_rn(c, d)), det);
    const float tu = __fdiv_rn(__fsub_rn(__fmul_rn(a, e), __fmul_rn(b, d)), det);
    s = clampf(su);
    t = clampf(tu);
    if (su < 0.f || su > 1.f) t = c > 0.f ? clampf(__fdiv_rn(__fadd_rn(__fmul_rn(b, s), e), c)) : 0.f;
    if (tu < 0.f || tu > 1.f) {
      s = a > 0.f ? clampf(__fdiv_rn(__fsub_rn(__fmul_rn(b, t), d), a)) : 0.f;
      t = c > 0.f ? clampf(__fdiv_rn(__fadd_rn(__fmul_rn(b, s), e), c)) : 0.f;
    }
  }
  float D[3];
  for (int q = 0; q < 3; ++q) D[q] = __fsub_rn(__fadd_rn(w3[q], __fmul_rn(s, a3[q])), __fmul_rn(t, b3[q]));
  return __fdiv_rn(__fsub_rn(__fsqrt_rn(dotf(D, D)), rsf), rsf);
}

// start[s] = the first row of the old table (sorted by (ea, eb)) whose ea >= s, s in [0, ne]
__global__ void k_table_seg_start(xk_pairs p, long long ne, int32_t* __restrict__ start) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s > ne) return;
  long long lo = 0, hi = p.n;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (p.ea[mid] < s) lo = mid + 1; else hi = mid;
  }
  start[s] = (int32_t)lo;
}

// Difference of two positions held as float hi/lo pairs (the node records): the hi and lo parts
// subtracted separately and then added, each operation rounded on its own.
XK_D float split_diff(const float* p, const float* q, int c) {
  return __fadd_rn(__fsub_rn(p[c], q[c]), __fsub_rn(p[3 + c], q[3 + c]));
}

__global__ void k_features(xk_mesh m, const float* __restrict__ n32, const int32_t* __restrict__ cands, long long n,
                           xk_pairs old, const int32_t* __restrict__ ostart, float* __restrict__ feat,
                           uint8_t* __restrict__ hist) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ea = cands[2 * i], eb = cands[2 * i + 1];
  const int nd[4] = {m.conn[2 * ea], m.conn[2 * ea + 1], m.conn[2 * eb], m.conn[2 * eb + 1]};
  float x[4][6];  // x_hi (3), x_lo (3) of the four nodes
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float4* r = reinterpret_cast<const float4*>(n32 + (long long)nd[k] * XK_NODE32_STRIDE);
    const float4 p = __ldg(r), q = __ldg(r + 1);
    x[k][0] = p.x; x[k][1] = p.y; x[k][2] = p.z; x[k][3] = p.w; x[k][4] = q.x; x[k][5] = q.y;
  }
  const float rsf = xk_d2f(xadd(m.radii[ea], m.radii[eb]));
  // position differences from the split records (no double arithmetic), then everything in float with
  // each operation rounded on its own
  float dm[3], da[3], db[3], dw[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    da[c] = split_diff(x[1], x[0], c);
    db[c] = split_diff(x[3], x[2], c);
    dw[c] = split_diff(x[0], x[2], c);
    // m_a - m_b = ((a0 - b0) + (a1 - b1)) / 2
    dm[c] = __fmul_rn(0.5f, __fadd_rn(dw[c], split_diff(x[1], x[3], c)));
  }
  auto dotf = [](const float* p, const float* q) {
    return __fadd_rn(__fadd_rn(__fmul_rn(p[0], q[0]), __fmul_rn(p[1], q[1])), __fmul_rn(p[2], q[2]));
  };
  const float sep = __fsqrt_rn(dotf(dm, dm));
  const float lna = __fsqrt_rn(dotf(da, da)), lnb = __fsqrt_rn(dotf(db, db));
  float den = __fmul_rn(lna, lnb);
  if (!(den >= 1e-30f)) den = (den != den) ? den : 1e-30f;
  float f[MF];
  f[0] = __fdiv_rn(sep, rsf);
  f[1] = __fdiv_rn(fabsf(dotf(da, db)), den);
  f[2] = __fdiv_rn(__fadd_rn(lna, lnb), __fmul_rn(2.0f, rsf));
  const int la = m.layer ? m.layer[ea] : -1, lb = m.layer ? m.layer[eb] : -1;
  const bool have = la >= 0 && lb >= 0;
  const int dl = la > lb ? la - lb : lb - la;
  f[3] = have ? __fdiv_rn((float)(dl < 3 ? dl : 3), 3.0f) : 0.f;
  f[4] = (have && (la == 0 || lb == 0)) ? 1.f : 0.f;
  // previous-step gap: the pair in the old table (sorted by (ea, eb)), searched among the rows of ea
  long long lo = ostart[ea], hi = (long long)ostart[ea + 1] - 1, at = -1;
  while (lo <= hi) {
    const long long mid = (lo + hi) >> 1;
    const int ob = old.eb[mid];
    if (ob == eb) { at = mid; break; }
    if (ob < eb) lo = mid + 1; else hi = mid - 1;
  }
  float g5;
  if (at >= 0) {
    g5 = __fdiv_rn((float)old.gap[at], rsf);
  } else {  // no previous gap: the current one, in float (feature accuracy is enough)
    g5 = current_gap_f(da, db, dw, rsf);
  }
  g5 = g5 < -2.0f ? -2.0f : (g5 > 8.0f ? 8.0f : g5);
  f[5] = g5;
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

// ------------------------------------------------------------------ inference (tcgen05, TMEM accumulators)
//
// One CTA of 128 threads per tile of 128 candidates, persistent over tiles.
// Operands live in shared memory in the canonical K-major layout without
// swizzle: 8-row x 16-byte core matrices (row r of a core at +16 r), cores
// adjacent along K LBO = 128 B apart, 8-row groups SBO apart.  Thread 0 issues
// tcgen05.mma (kind::f16, BF16 in, FP32 accumulate, M 128, N 64, K 16 per
// instruction) into a 64-column TMEM accumulator and commits to an mbarrier;
// the four warps read their 32 lanes (rows) back with tcgen05.ld, add the bias,
// apply ReLU, round to BF16 and write the next layer's operand tile.
// Every wait is bounded: on expiry the kernel sets *err, skips the remaining
// work, and still frees its TMEM.

constexpr int TC_T = 128;
constexpr int TC_PER_SM = 5;
constexpr uint32_t TC_COLS = 64;
// instruction descriptor: D f32 (bit 4), A bf16 (bits 7-9 = 1), B bf16 (bits 10-12 = 1),
// K-major A and B (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
constexpr long long TC_SPIN = 1LL << 22;

XK_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start >> 4 (bits 0-13), LBO >> 4 (16-29), SBO >> 4 (32-45),
// fixed 0b001 at bits 46-48, no base offset, relative LBO, no swizzle (bits 61-63 = 0)
XK_D uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

XK_D void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
      :
      : "r"(dtmem), "l"(adesc), "l"(bdesc), "r"(TC_IDESC), "r"(accumulate));
}

XK_D void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}

// bounded wait for the mbarrier phase `parity`; false on expiry
XK_D bool tc_wait(uint32_t mbar, uint32_t parity) {
  for (long long it = 0; it < TC_SPIN; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 16 consecutive fp32 columns of this thread's TMEM lane
XK_D void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

XK_D void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
XK_D void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
XK_D void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
XK_D void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// byte offset of element (row, k) (16-bit elements) in a K-major no-swizzle tile with K columns
XK_D uint32_t core_off(int row, int k, int K) {
  return (uint32_t)((row >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// The biases ride in the MMAs: layer 1's operand has a constant-one column
// (k = 8) matched by b1 in W1's padding, and layers 2 and 3 add one K-16 MMA
// of a constant tile (column 0 = 1) against a bias tile (column 0 = b).  The
// BF16 biases times 1 are exact in the FP32 accumulator.
struct __align__(128) TcSmem {
  // hidden operand (layers 2 and 3); its first 4 KB also hold the layer-1 operand
  // (128 candidates x K 16: 8 features, 1, 7 zeros), read only before the hidden
  // operand is first written for the tile
  uint16_t a2[128 * 64];
  uint16_t ones[128 * 16];  // 128 x K 16, column 0 = 1
  uint16_t w1[64 * 16];     // [W1 | b1 | 0] as N 64 x K 16
  uint16_t w2[64 * 64];
  uint16_t w3[64 * 64];
  uint16_t bb2[64 * 16];    // column 0 = b2
  uint16_t bb3[64 * 16];    // column 0 = b3
  float w4[64];
  float b4;
  uint64_t mbar;
  uint32_t tmem;
};

// two floats -> bf16x2 (lo in the low half), each max(x, 0) rounded to nearest even
XK_D uint32_t pack_relu_bf16(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;\n" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}

__global__ void __launch_bounds__(TC_T) k_mlp_forward_tc(const uint16_t* __restrict__ P,
                                                         const float* __restrict__ feat, long long n,
                                                         float* __restrict__ logit, int* __restrict__ err) {
  __shared__ TcSmem sm;
  const int tid = threadIdx.x, warp = tid >> 5;
  // weights in the operand layout (N rows = outputs, K = inputs), biases as float
  constexpr uint16_t BF16_ONE = 0x3F80;
  for (int i = tid; i < 64 * 16; i += TC_T) {
    const int nn = i >> 4, k = i & 15;
    const uint16_t v = k < MF ? P[O_W1 + nn * MF + k] : k == MF ? P[O_B1 + nn] : (uint16_t)0;
    const uint32_t o = core_off(nn, k, 16);
    *reinterpret_cast<uint16_t*>(reinterpret_cast<char*>(sm.w1) + o) = v;
    *reinterpret_cast<uint16_t*>(reinterpret_cast<char*>(sm.bb2) + o) = k == 0 ? P[O_B2 + nn] : (uint16_t)0;
    *reinterpret_cast<uint16_t*>(reinterpret_cast<char*>(sm.bb3) + o) = k == 0 ? P[O_B3 + nn] : (uint16_t)0;
  }
  for (int i = tid; i < 128 * 16; i += TC_T) {
    const int r = i >> 4, k = i & 15;
    *reinterpret_cast<uint16_t*>(reinterpret_cast<char*>(sm.ones) + core_off(r, k, 16)) =
        k == 0 ? BF16_ONE : (uint16_t)0;
  }
  // W2, W3: one 16-byte core-matrix row (8 consecutive k of output nn) per copy; the
  // parameter offsets of both are multiples of 8 elements
  static_assert(O_W2 % 8 == 0 && O_W3 % 8 == 0, "16-byte weight rows");
  for (int i = tid; i < 64 * 8; i += TC_T) {
    const int nn = i >> 3, kc = i & 7;
    const uint32_t o = core_off(nn, 8 * kc, 64);
    *reinterpret_cast<uint4*>(reinterpret_cast<char*>(sm.w2) + o) = *reinterpret_cast<const uint4*>(P + O_W2 + 8 * i);
    *reinterpret_cast<uint4*>(reinterpret_cast<char*>(sm.w3) + o) = *reinterpret_cast<const uint4*>(P + O_W3 + 8 * i);
  }
  if (tid < 64) sm.w4[tid] = bf16_at(P, O_W4 + tid);
  if (tid == 0) {
    sm.b4 = bf16_at(P, O_B4);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&sm.mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&sm.tmem)),
                 "r"(TC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem;
  const uint32_t mbar = smem_u32(&sm.mbar);
  const uint32_t lane_base = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's 32 TMEM lanes
  uint32_t phase = 0;
  bool ok = true;
  const long long tiles = (n + 127) / 128;
  // features of this thread's row of a tile (zero beyond n); the next tile's are loaded while
  // the current tile runs its layers
  auto load_row = [&](long long tile, float4& lo, float4& hi) {
    const long long row = tile * 128 + tid;
    if (tile < tiles && row < n) {
      const float4* f4 = reinterpret_cast<const float4*>(feat + MF * row);
      lo = __ldcs(f4);
      hi = __ldcs(f4 + 1);
    } else {
      lo = hi = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };
  float4 x_lo, x_hi;
  load_row(blockIdx.x, x_lo, x_hi);
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const long long row = tile * 128 + tid;  // thread tid owns tile row tid (its TMEM lane)
    {  // layer-1 operand: the features rounded to bf16, the one for b1, zeros
      uint4 v0, v1;
      v0.x = pack_bf16(x_lo.x, x_lo.y); v0.y = pack_bf16(x_lo.z, x_lo.w);
      v0.z = pack_bf16(x_hi.x, x_hi.y); v0.w = pack_bf16(x_hi.z, x_hi.w);
      v1.x = BF16_ONE;  // k = 8: the constant-one column that carries b1
      v1.y = v1.z = v1.w = 0u;
      *reinterpret_cast<uint4*>(reinterpret_cast<char*>(sm.a2) + core_off(tid, 0, 16)) = v0;
      *reinterpret_cast<uint4*>(reinterpret_cast<char*>(sm.a2) + core_off(tid, 8, 16)) = v1;
    }
    load_row(tile + gridDim.x, x_lo, x_hi);
    float out = 0.f;
#pragma unroll 1
    for (int layer = 0; layer < 3 && ok; ++layer) {
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (tid == 0) {
        if (layer == 0) {
          tc_mma(tmem, tc_desc(smem_u32(sm.a2), 128, 256), tc_desc(smem_u32(sm.w1), 128, 256), 0u);
        } else {
          const uint16_t* w = layer == 1 ? sm.w2 : sm.w3;
#pragma unroll
          for (int ks = 0; ks < 4; ++ks)
            tc_mma(tmem, tc_desc(smem_u32(sm.a2) + ks * 256, 128, 1024), tc_desc(smem_u32(w) + ks * 256, 128, 1024),
                   ks > 0 ? 1u : 0u);
          tc_mma(tmem, tc_desc(smem_u32(sm.ones), 128, 256), tc_desc(smem_u32(layer == 1 ? sm.bb2 : sm.bb3), 128, 256),
                 1u);
        }
        tc_commit(mbar);
      }
      // the outcome of the wait is made uniform over the block before anyone acts on it
      if (__syncthreads_or(tc_wait(mbar, phase) ? 0 : 1)) {
        ok = false;
        break;
      }
      phase ^= 1u;
      tc_fence_after();
      // the MMA that read the operand tile has completed, so the next operand is written in
      // place; the next MMA is issued only after the barrier at the top of the layer loop,
      // which every thread reaches after its tcgen05.ld has retired
      float z[64];
      tc_ld16(lane_base + 0, z);
      tc_ld16(lane_base + 16, z + 16);
      tc_ld16(lane_base + 32, z + 32);
      tc_ld16(lane_base + 48, z + 48);
      tc_wait_ld();
      if (layer < 2) {
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          uint4 v;
          v.x = pack_relu_bf16(z[8 * c + 0], z[8 * c + 1]);
          v.y = pack_relu_bf16(z[8 * c + 2], z[8 * c + 3]);
          v.z = pack_relu_bf16(z[8 * c + 4], z[8 * c + 5]);
          v.w = pack_relu_bf16(z[8 * c + 6], z[8 * c + 7]);
          *reinterpret_cast<uint4*>(reinterpret_cast<char*>(sm.a2) + core_off(tid, 8 * c, 64)) = v;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 64; j += 2) {
          const uint32_t h = pack_relu_bf16(z[j], z[j + 1]);
          out = fmaf(__uint_as_float(h << 16), sm.w4[j], out);
          out = fmaf(__uint_as_float(h & 0xFFFF0000u), sm.w4[j + 1], out);
        }
      }
      if (layer == 2) out += sm.b4;
    }
    if (ok && row < n) logit[row] = out;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
  if (!ok && tid == 0) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_COLS) : "memory");
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

// keep flag of candidate i; a scoring that reported an expired tensor-core wait (*err != 0) keeps every
// candidate, since its scores are undefined
__global__ void k_keep_flags(long long n, const float* __restrict__ logit, const uint8_t* __restrict__ hist,
                             float thr, int invert, const int32_t* __restrict__ err, int32_t* __restrict__ flag) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const int keep = (logit[i] >= thr || (hist && hist[i]) || (err && *err)) ? 1 : 0;
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

extern "C" xk_status xk_prune_features(const xk_mesh* m, const float* node32, const int32_t* cands, int64_t n,
                                       const xk_pairs* old, float* feat, uint8_t* hist, xk_stream s) {
  if (!m || !old || (n > 0 && (!cands || !feat || !hist || !node32)) || n < 0)
    return xk_set_error(XK_ERR_ARG, "xk_prune_features: bad arguments");
  if (n == 0) return XK_OK;
  cudaStream_t st = (cudaStream_t)s;
  const long long ne = m->n_elems;
  int32_t* ostart = nullptr;
  XK_CUDA(cudaMallocAsync((void**)&ostart, sizeof(int32_t) * (ne + 2), st));
  k_table_seg_start<<<xk_blocks(ne + 1, 256), 256, 0, st>>>(*old, ne, ostart);
  k_features<<<xk_blocks(n, 256), 256, 0, st>>>(*m, node32, cands, n, *old, ostart, feat, hist);
  cudaError_t e = cudaGetLastError();
  cudaFreeAsync(ostart, st);
  if (e != cudaSuccess) return xk_set_cuda_error(e, __FILE__, __LINE__);
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

extern "C" xk_status xk_mlp_forward_tcgen05(const uint16_t* params_bf16, const float* feat, int64_t n, float* logit,
                                            int* err, xk_stream s) {
  if (!params_bf16 || !err || n < 0 || (n > 0 && (!feat || !logit)))
    return xk_set_error(XK_ERR_ARG, "xk_mlp_forward_tcgen05: bad arguments");
  if ((reinterpret_cast<uintptr_t>(params_bf16) & 15) || (reinterpret_cast<uintptr_t>(feat) & 15))
    return xk_set_error(XK_ERR_ARG, "xk_mlp_forward_tcgen05: params and feat must be 16-byte aligned");
  if (n == 0) return XK_OK;
  // persistent grid of TC_PER_SM CTAs per SM: each CTA runs its tiles' three layers back to back
  // (MMA, completion wait, read-back), so several CTAs per SM overlap one's MMA with another's
  // read-back; five measured best on 400k-8M samples (4 to 8 within 15%)
  const int sms = xk_sm_count();
  const long long resident = (long long)TC_PER_SM * sms;
  const long long tiles = (n + 127) / 128;
  const int blocks = (int)(tiles < resident ? tiles : resident);
  k_mlp_forward_tc<<<blocks, TC_T, 0, (cudaStream_t)s>>>(params_bf16, feat, n, logit, err);
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
                                     float threshold, int invert, const int32_t* score_error, int32_t* kept,
                                     int64_t* n_kept, int32_t* score_failed, xk_stream s) {
  if (!n_kept || n < 0 || (n > 0 && (!cands || !logit || !kept)))
    return xk_set_error(XK_ERR_ARG, "xk_prune_select: bad arguments");
  *n_kept = 0;
  if (score_failed) *score_failed = 0;
  if (n == 0) return XK_OK;
  cudaStream_t st = (cudaStream_t)s;
  int32_t* flag = nullptr;
  int64_t* tot = nullptr;  // [count, scoring error word]
  XK_CUDA(cudaMallocAsync((void**)&flag, sizeof(int32_t) * 2 * n, st));
  cudaError_t e = cudaMallocAsync((void**)&tot, 2 * sizeof(int64_t), st);
  if (e != cudaSuccess) {
    cudaFreeAsync(flag, st);
    return xk_set_cuda_error(e, __FILE__, __LINE__);
  }
  int32_t* off = flag + n;
  k_keep_flags<<<xk_blocks(n, 256), 256, 0, st>>>(n, logit, hist, threshold, invert, score_error, flag);
  xk_status r = xk_exclusive_scan_i32(flag, off, n, tot, st);
  if (r == XK_OK) {
    k_scatter_cands<<<xk_blocks(n, 256), 256, 0, st>>>(n, cands, flag, off, kept);
    int64_t h[2] = {0, 0};
    e = cudaGetLastError();
    // the count and the scoring's error word come back in one copy
    if (e == cudaSuccess && score_error)
      e = cudaMemcpyAsync(tot + 1, score_error, sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, tot, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      r = xk_set_cuda_error(e, __FILE__, __LINE__);
    } else {
      *n_kept = h[0];
      if (score_failed && score_error) *score_failed = (int32_t)(h[1] & 0xffffffff);
    }
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
