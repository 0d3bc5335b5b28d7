// Error state, device-wide scans, radix sort and FP64 reductions.
#include <atomic>
#include <cstdio>
#include <cstring>

#include "xk_common.cuh"

static thread_local char g_err[512] = "";

extern "C" const char* xk_version(void) { return "xkgpu 0.1 (sm_103a)"; }
extern "C" const char* xk_last_error(void) { return g_err; }

xk_status xk_set_cuda_error(cudaError_t e, const char* file, int line) {
  snprintf(g_err, sizeof(g_err), "CUDA error %d (%s) at %s:%d", (int)e, cudaGetErrorString(e), file, line);
  return XK_ERR_CUDA;
}
xk_status xk_set_error(xk_status code, const char* msg) {
  snprintf(g_err, sizeof(g_err), "%s", msg);
  return code;
}

int xk_sm_count() {
  constexpr int MAX_DEV = 64;
  static std::atomic<int> cache[MAX_DEV];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
  if (dev >= MAX_DEV) {
    int n = 0;
    return (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0) ? n : 1;
  }
  int n = cache[dev].load(std::memory_order_relaxed);
  if (n > 0) return n;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
  cache[dev].store(n, std::memory_order_relaxed);
  return n;
}

// --------------------------------------------------------------------------- scan

namespace {
constexpr int SCAN_T = 256;
constexpr int SCAN_I = 8;
constexpr int SCAN_TILE = SCAN_T * SCAN_I;

template <typename T>
__device__ T block_exclusive_scan(T v, T* warp_tot, T* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = (lane < (SCAN_T / 32)) ? warp_tot[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < (SCAN_T / 32)) warp_tot[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  T before = (warp > 0) ? warp_tot[warp - 1] : T(0);
  if (total) *total = warp_tot[SCAN_T / 32 - 1];
  return before + x - v;
}

template <typename TI>
__global__ void k_tile_sums(const TI* __restrict__ in, long long n, int64_t* __restrict__ bsum) {
  __shared__ int64_t wt[SCAN_T / 32];
  long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_I;
  int64_t s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_I; ++i)
    if (base + i < n) s += (int64_t)in[base + i];
  int64_t tot;
  block_exclusive_scan<int64_t>(s, wt, &tot);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void k_scan_bsums(int64_t* bsum, long long nb, int64_t* total) {
  __shared__ int64_t wt[SCAN_T / 32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (long long b0 = 0; b0 < nb; b0 += SCAN_T) {
    long long i = b0 + threadIdx.x;
    int64_t v = (i < nb) ? bsum[i] : 0;
    int64_t tot;
    int64_t ex = block_exclusive_scan<int64_t>(v, wt, &tot);
    int64_t c = carry;
    if (i < nb) bsum[i] = c + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry = c + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

template <typename TI, typename TO>
__global__ void k_tile_scan(const TI* __restrict__ in, TO* __restrict__ out, long long n,
                            const int64_t* __restrict__ bsum) {
  __shared__ int64_t wt[SCAN_T / 32];
  long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_I;
  int64_t loc[SCAN_I];
  int64_t s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_I; ++i) {
    loc[i] = (base + i < n) ? (int64_t)in[base + i] : 0;
    s += loc[i];
  }
  int64_t ex = block_exclusive_scan<int64_t>(s, wt, nullptr) + bsum[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_I; ++i) {
    if (base + i < n) out[base + i] = (TO)ex;
    ex += loc[i];
  }
}

// One-pass scan with decoupled look-back (Merrill and Garland, "Single-pass Parallel Prefix Scan with
// Decoupled Look-back", NVIDIA technical report NVR-2016-002).  Tiles take their index from a ticket
// counter in the order they start, so a tile waits only on tiles that are already running and never on a
// later one.  Each tile publishes its aggregate (flag 1); the first warp then looks back over a window of
// 32 predecessors at a time (one flag per lane, ballots to find the nearest inclusive prefix, flag 2, and
// any predecessor that has not published), adds the window's aggregates up to that prefix with a warp sum,
// and publishes the tile's inclusive prefix.  The wait on a predecessor that has not published yet is
// bounded: past SCAN_SPIN_LIMIT polls the tile sums the inputs before it itself (the same prefix: integer
// sums do not depend on their order), so the result never depends on the wait.
constexpr int SCAN_SPIN_LIMIT = 1 << 20;

XK_D int ld_flag(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}

// Eight consecutive inputs of one thread; 32-bit inputs at a 16-byte aligned address as two vector loads.
template <typename TI>
XK_D void load_tile8(const TI* __restrict__ in, long long base, long long n, int64_t* loc) {
  if (sizeof(TI) == 4 && base + SCAN_I <= n && ((reinterpret_cast<uintptr_t>(in + base) & 15) == 0)) {
    const int4* q = reinterpret_cast<const int4*>(in + base);
    const int4 x = __ldg(q), y = __ldg(q + 1);
    loc[0] = x.x; loc[1] = x.y; loc[2] = x.z; loc[3] = x.w;
    loc[4] = y.x; loc[5] = y.y; loc[6] = y.z; loc[7] = y.w;
    return;
  }
#pragma unroll
  for (int i = 0; i < SCAN_I; ++i) loc[i] = (base + i < n) ? (int64_t)in[base + i] : 0;
}

template <typename TI, typename TO>
__global__ void __launch_bounds__(SCAN_T) k_scan_onepass(const TI* __restrict__ in, TO* __restrict__ out,
                                                         long long n, long long nb, int64_t* __restrict__ total,
                                                         int64_t* __restrict__ agg, int64_t* __restrict__ inc,
                                                         int* __restrict__ flag, unsigned* __restrict__ ticket) {
  __shared__ int64_t wt[SCAN_T / 32];
  __shared__ long long s_tile;
  __shared__ int64_t s_prefix;
  __shared__ int s_fallback;
  if (threadIdx.x == 0) {
    s_tile = (long long)atomicAdd(ticket, 1u);
    s_fallback = 0;
  }
  __syncthreads();
  const long long t = s_tile;
  const long long base = t * SCAN_TILE + (long long)threadIdx.x * SCAN_I;
  int64_t loc[SCAN_I];
  load_tile8<TI>(in, base, n, loc);
  int64_t s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_I; ++i) s += loc[i];
  int64_t tile_tot;
  int64_t ex = block_exclusive_scan<int64_t>(s, wt, &tile_tot);
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    if (t == 0) {
      if (lane == 0) {
        inc[0] = tile_tot;
        __threadfence();
        atomicExch(&flag[0], 2);
        s_prefix = 0;
      }
    } else {
      if (lane == 0) {
        agg[t] = tile_tot;
        __threadfence();
        atomicExch(&flag[t], 1);
      }
      int64_t p = 0;
      long long j = t - 1;  // the window covers tiles j, j - 1, ..., j - 31 (lane k: tile j - k)
      int spins = 0;
      bool fell_back = false;
      while (true) {
        const long long k = j - lane;
        const int f = k >= 0 ? ld_flag(flag + k) : 2;  // before tile 0: an inclusive prefix of 0
        const unsigned m_inc = __ballot_sync(0xffffffffu, f == 2);
        const int stop = m_inc ? __ffs(m_inc) - 1 : 32;  // nearest inclusive prefix in the window
        const unsigned need = stop == 32 ? 0xffffffffu : ((1u << stop) - 1u);
        if (__ballot_sync(0xffffffffu, f == 0) & need) {  // a nearer predecessor has not published
          if (++spins > SCAN_SPIN_LIMIT) {
            fell_back = true;
            break;
          }
          continue;
        }
        __threadfence();
        // published values are read past L1 (other tiles' lines may sit there stale)
        int64_t v = 0;
        if (k >= 0) {
          if (lane < stop) v = __ldcg(agg + k);
          else if (lane == stop) v = __ldcg(inc + k);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        p += v;
        if (stop < 32) break;
        j -= 32;
      }
      if (lane == 0) {
        if (fell_back) {
          s_fallback = 1;
        } else {
          inc[t] = p + tile_tot;
          __threadfence();
          atomicExch(&flag[t], 2);
          s_prefix = p;
        }
      }
    }
  }
  __syncthreads();
  if (s_fallback) {  // the prefix from the inputs before this tile
    int64_t q = 0;
    for (long long k = threadIdx.x; k < t * SCAN_TILE; k += SCAN_T) q += (int64_t)in[k];
    int64_t all;
    block_exclusive_scan<int64_t>(q, wt, &all);
    if (threadIdx.x == 0) {
      s_prefix = all;
      inc[t] = all + tile_tot;
      __threadfence();
      atomicExch(&flag[t], 2);
    }
    __syncthreads();
  }
  ex += s_prefix;
#pragma unroll
  for (int i = 0; i < SCAN_I; ++i) {
    if (base + i < n) out[base + i] = (TO)ex;
    ex += loc[i];
  }
  if (t == nb - 1 && threadIdx.x == 0 && total) *total = s_prefix + tile_tot;
}

template <typename TI, typename TO>
xk_status scan_impl(const TI* in, TO* out, long long n, int64_t* total_dev, cudaStream_t s) {
  if (n <= 0) {
    if (total_dev) XK_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(int64_t), s));
    return XK_OK;
  }
  const long long nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  // one allocation: aggregates, inclusive prefixes, then the flags and the ticket (zeroed)
  char* buf = nullptr;
  const size_t words = sizeof(int64_t) * 2 * nb, tail = sizeof(int) * (nb + 1);
  XK_CUDA(cudaMallocAsync((void**)&buf, words + tail, s));
  int64_t* agg = reinterpret_cast<int64_t*>(buf);
  int* flag = reinterpret_cast<int*>(buf + words);
  cudaError_t e = cudaMemsetAsync(flag, 0, tail, s);
  if (e == cudaSuccess) {
    k_scan_onepass<TI, TO><<<(unsigned)nb, SCAN_T, 0, s>>>(in, out, n, nb, total_dev, agg, agg + nb, flag,
                                                           reinterpret_cast<unsigned*>(flag + nb));
    e = cudaGetLastError();
  }
  cudaFreeAsync(buf, s);
  if (e != cudaSuccess) return xk_set_cuda_error(e, __FILE__, __LINE__);
  return XK_OK;
}
}  // namespace

xk_status xk_exclusive_scan_i32(const int32_t* in, int32_t* out, long long n, int64_t* total_dev,
                                cudaStream_t s) {
  return scan_impl<int32_t, int32_t>(in, out, n, total_dev, s);
}
xk_status xk_exclusive_scan_i64(const int64_t* in, int64_t* out, long long n, int64_t* total_dev,
                                cudaStream_t s) {
  return scan_impl<int64_t, int64_t>(in, out, n, total_dev, s);
}

long long xk_scan_tiles(long long n) { return n <= 0 ? 0 : (n + SCAN_TILE - 1) / SCAN_TILE; }

xk_status xk_exclusive_scan_i32_scratch(const int32_t* in, int32_t* out, long long n, int64_t* total_dev,
                                        int64_t* bsum, long long bsum_cap, cudaStream_t s) {
  if (n <= 0) {
    if (total_dev) XK_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(int64_t), s));
    return XK_OK;
  }
  long long nb = xk_scan_tiles(n);
  if (!bsum || nb > bsum_cap) return xk_set_error(XK_ERR_CAPACITY, "scan: block-sum scratch too small");
  k_tile_sums<int32_t><<<(unsigned)nb, SCAN_T, 0, s>>>(in, n, bsum);
  k_scan_bsums<<<1, SCAN_T, 0, s>>>(bsum, nb, total_dev);
  k_tile_scan<int32_t, int32_t><<<(unsigned)nb, SCAN_T, 0, s>>>(in, out, n, bsum);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

// --------------------------------------------------------------------------- radix sort

namespace {
constexpr int RS_T = 256;
constexpr int RS_I = 8;
constexpr int RS_TILE = RS_T * RS_I;

__global__ void k_rs_hist(const uint64_t* __restrict__ keys, long long n, int shift,
                          int32_t* __restrict__ hist, int nblocks) {
  __shared__ int cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  long long t0 = (long long)blockIdx.x * RS_TILE;
  for (int i = 0; i < RS_I; ++i) {
    long long idx = t0 + (long long)i * RS_T + threadIdx.x;
    if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & 255u], 1);
  }
  __syncthreads();
  hist[(long long)threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void k_rs_scatter(const uint64_t* __restrict__ kin, const int32_t* __restrict__ vin,
                             uint64_t* __restrict__ kout, int32_t* __restrict__ vout, long long n,
                             int shift, const int32_t* __restrict__ off, int nblocks) {
  __shared__ int run[256];
  run[threadIdx.x] = off[(long long)threadIdx.x * nblocks + blockIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  long long t0 = (long long)blockIdx.x * RS_TILE;
  for (int i = 0; i < RS_I; ++i) {
    long long idx = t0 + (long long)i * RS_T + threadIdx.x;
    bool valid = idx < n;
    uint64_t k = valid ? kin[idx] : 0ull;
    int32_t v = valid ? vin[idx] : 0;
    int d = valid ? (int)((k >> shift) & 255u) : 256;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    int rank = __popc(peers & lt);
    int cntw = __popc(peers);
    int leader = __ffs(peers) - 1;
    for (int w = 0; w < RS_T / 32; ++w) {
      __syncthreads();
      if (warp == w) {
        int base = (lane == leader && valid) ? run[d] : 0;
        base = __shfl_sync(0xffffffffu, base, leader);
        if (valid) {
          long long dst = (long long)base + rank;
          kout[dst] = k;
          vout[dst] = v;
        }
        if (lane == leader && valid) run[d] = base + cntw;
      }
    }
    __syncthreads();
  }
}
}  // namespace

xk_status xk_radix_sort_u64(uint64_t* keys, int32_t* vals, long long n, int bits, cudaStream_t s) {
  if (n <= 1) return XK_OK;
  int passes = (bits + 7) / 8;
  if (passes <= 0) return XK_OK;
  int nb = (int)((n + RS_TILE - 1) / RS_TILE);
  uint64_t* k2 = nullptr;
  int32_t *v2 = nullptr, *hist = nullptr;
  XK_CUDA(cudaMallocAsync((void**)&k2, sizeof(uint64_t) * n, s));
  XK_CUDA(cudaMallocAsync((void**)&v2, sizeof(int32_t) * n, s));
  XK_CUDA(cudaMallocAsync((void**)&hist, sizeof(int32_t) * 256 * (long long)nb, s));
  uint64_t *ka = keys, *kb = k2;
  int32_t *va = vals, *vb = v2;
  xk_status st = XK_OK;
  for (int p = 0; p < passes && st == XK_OK; ++p) {
    int shift = 8 * p;
    k_rs_hist<<<nb, RS_T, 0, s>>>(ka, n, shift, hist, nb);
    st = xk_exclusive_scan_i32(hist, hist, 256LL * nb, nullptr, s);
    if (st != XK_OK) break;
    k_rs_scatter<<<nb, RS_T, 0, s>>>(ka, va, kb, vb, n, shift, hist, nb);
    uint64_t* tk = ka; ka = kb; kb = tk;
    int32_t* tv = va; va = vb; vb = tv;
  }
  cudaError_t e = cudaGetLastError();
  if (st == XK_OK && e == cudaSuccess && ka != keys) {
    e = cudaMemcpyAsync(keys, ka, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(vals, va, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s);
  }
  cudaFreeAsync(k2, s);
  cudaFreeAsync(v2, s);
  cudaFreeAsync(hist, s);
  if (st != XK_OK) return st;
  if (e != cudaSuccess) return xk_set_cuda_error(e, __FILE__, __LINE__);
  return XK_OK;
}

// --------------------------------------------------------------------------- FP64 sum of squares

namespace {
constexpr int N2_BLOCKS = 304;  // 2 x 152 SMs; fixed so that the summation order is fixed
constexpr int N2_T = 256;

__global__ void k_sumsq_partial(const double* __restrict__ x, long long n, double* __restrict__ part) {
  __shared__ double sm[N2_T];
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * N2_T + threadIdx.x; i < n; i += (long long)N2_BLOCKS * N2_T)
    acc = fma(x[i], x[i], acc);
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int w = N2_T / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

__global__ void k_sum_final(const double* __restrict__ part, int np, double* __restrict__ out) {
  __shared__ double sm[512];
  double a = 0.0;
  for (int i = threadIdx.x; i < np; i += 512) a += part[i];
  sm[threadIdx.x] = a;
  __syncthreads();
  for (int w = 256; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0];
}
}  // namespace

// Partials buffer for the fixed-order reductions; one per device, set up on the
// first call (cudaMalloc outside any capture).
static double* g_part[64] = {nullptr};

xk_status xk_partials_buffer(double** out) {
  int dev = 0;
  XK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return xk_set_error(XK_ERR_ARG, "device ordinal out of range");
  if (!g_part[dev]) XK_CUDA(cudaMalloc((void**)&g_part[dev], sizeof(double) * N2_BLOCKS));
  *out = g_part[dev];
  return XK_OK;
}

xk_status xk_sumsq_into(const double* x, long long n, double* out, cudaStream_t s) {
  double* part = nullptr;
  xk_status st = xk_partials_buffer(&part);
  if (st != XK_OK) return st;
  k_sumsq_partial<<<N2_BLOCKS, N2_T, 0, s>>>(x, n, part);
  k_sum_final<<<1, 512, 0, s>>>(part, N2_BLOCKS, out);
  XK_CHECK_LAUNCH();
  return XK_OK;
}

extern "C" xk_status xk_norm2(const double* x, int64_t n, double* out, xk_stream s) {
  if (!x || !out || n < 0) return xk_set_error(XK_ERR_ARG, "xk_norm2: bad arguments");
  return xk_sumsq_into(x, n, out, (cudaStream_t)s);
}
