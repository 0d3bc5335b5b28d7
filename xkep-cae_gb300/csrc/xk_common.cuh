// Shared device/host helpers for the xkgpu kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xkgpu.h"

#define XK_HD __host__ __device__ __forceinline__
#define XK_D __device__ __forceinline__

// ---------------------------------------------------------------------------
// Exactly rounded double operations.  The parts of the path whose results are
// compared bit for bit with the reference (AABBs, closest point, gap, active
// set, midpoint prescreen) use these so that nvcc cannot contract a*b+c into
// an FMA; the reference's NumPy arithmetic rounds every product and sum.
// ---------------------------------------------------------------------------
#ifdef __CUDA_ARCH__
XK_D double xadd(double a, double b) { return __dadd_rn(a, b); }
XK_D double xsub(double a, double b) { return __dsub_rn(a, b); }
XK_D double xmul(double a, double b) { return __dmul_rn(a, b); }
XK_D double xdiv(double a, double b) { return __ddiv_rn(a, b); }
XK_D double xsqrt(double a) { return __dsqrt_rn(a); }
#else
inline double xadd(double a, double b) { return a + b; }
inline double xsub(double a, double b) { return a - b; }
inline double xmul(double a, double b) { return a * b; }
inline double xdiv(double a, double b) { return a / b; }
inline double xsqrt(double a) { return sqrt(a); }
#endif

// einsum('ij,ij->i') order measured for the reference's NumPy: (p0 + p2) + p1
XK_HD double xdot_es(const double* a, const double* b) {
  return xadd(xadd(xmul(a[0], b[0]), xmul(a[2], b[2])), xmul(a[1], b[1]));
}
// np.sum(axis=1) / np.linalg.norm order: (p0 + p1) + p2
XK_HD double xdot_seq(const double* a, const double* b) {
  return xadd(xadd(xmul(a[0], b[0]), xmul(a[1], b[1])), xmul(a[2], b[2]));
}
XK_HD void xcross(const double* a, const double* b, double* c) {
  c[0] = xsub(xmul(a[1], b[2]), xmul(a[2], b[1]));
  c[1] = xsub(xmul(a[2], b[0]), xmul(a[0], b[2]));
  c[2] = xsub(xmul(a[0], b[1]), xmul(a[1], b[0]));
}
// np.clip(x, 0, 1): NaN propagates
XK_HD double xclip01(double x) { return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x); }

// ---------------------------------------------------------------------------
// Generic small-vector helpers for the non-exact (FP64 plain or FP32 mixed) math.
// ---------------------------------------------------------------------------
template <typename T>
XK_HD T dot3(const T* a, const T* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <typename T>
XK_HD void cross3(const T* a, const T* b, T* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

template <typename T>
XK_HD T my_sqrt(T x);
template <>
XK_HD double my_sqrt<double>(double x) { return sqrt(x); }
template <>
XK_HD float my_sqrt<float>(float x) { return sqrtf(x); }
template <typename T>
XK_HD T my_abs(T x) { return x < T(0) ? -x : x; }

// Precision policy: P == XK_FP64 computes everything in double; P == XK_MIXED
// computes the bulk in float and keeps the rotation frames, the axial strain,
// the contact gap and all reductions in double.
template <int P>
struct Prec;
template <>
struct Prec<XK_FP64> { typedef double T; };
template <>
struct Prec<XK_MIXED> { typedef float T; };

// Double <-> float conversions in integer arithmetic.  On this GPU the conversion instructions issue
// at the FP64 rate (about 1.8 per clock per SM, like a double add, against about 100 float adds),
// and the integer operations at the full rate.  Both give the bits of the IEEE conversion (round to
// nearest, ties to even, for double -> float; exact for float -> double): the fields are moved as
// integers, and a result or input that is not a normal number (denormal, overflow, inf, nan) takes
// the conversion instruction.
XK_D float xk_d2f(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned e = (hi >> 20) & 0x7ffu;  // biased exponent; a normal float result needs e in [897, 1150]
  if (e - 897u > 253u) {
    if (((hi & 0x7fffffffu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);  // +-0
    return __double2float_rn(x);
  }
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // the top 23 of the 52 mantissa bits
  const unsigned r = lo & 0x1fffffffu;                     // the 29 bits rounded away
  const unsigned up = (r > 0x10000000u || (r == 0x10000000u && (m & 1u))) ? 1u : 0u;
  // a carry out of the mantissa raises the exponent (and past the largest float gives inf), as rounding does
  return __uint_as_float(((hi & 0x80000000u) | ((e - 896u) << 23) | m) + up);
}
XK_D double xk_f2d(float v) {
  const unsigned f = __float_as_uint(v);
  const unsigned e = (f >> 23) & 0xffu;
  if (e - 1u > 253u) {
    if ((f & 0x7fffffffu) == 0u) return __hiloint2double((int)(f & 0x80000000u), 0);  // +-0
    return (double)v;
  }
  return __hiloint2double((int)((f & 0x80000000u) | ((e + 896u) << 20) | ((f & 0x7fffffu) >> 3)), (int)(f << 29));
}

// Eight floats from a 32-byte aligned read-only address in one 256-bit load.
XK_D void ldg8(const float* __restrict__ p, float* v) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
      : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
      : "l"(p));
}

// ---------------------------------------------------------------------------
// Launch helpers
// ---------------------------------------------------------------------------
static inline int xk_blocks(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 0x7fffffffLL) b = 0x7fffffffLL;
  return (int)b;
}

#define XK_CHECK_LAUNCH()                                      \
  do {                                                         \
    cudaError_t e__ = cudaGetLastError();                      \
    if (e__ != cudaSuccess) return xk_set_cuda_error(e__, __FILE__, __LINE__); \
  } while (0)

#define XK_CUDA(call)                                          \
  do {                                                         \
    cudaError_t e__ = (call);                                  \
    if (e__ != cudaSuccess) return xk_set_cuda_error(e__, __FILE__, __LINE__); \
  } while (0)

xk_status xk_set_cuda_error(cudaError_t e, const char* file, int line);
xk_status xk_set_error(xk_status code, const char* msg);

// SM count of the current device, read once per device ordinal (1 when it cannot be read).
int xk_sm_count();

// Device-wide exclusive scans (scan.cu).  Scratch is allocated stream-ordered.
xk_status xk_exclusive_scan_i32(const int32_t* in, int32_t* out, long long n, int64_t* total_dev,
                                cudaStream_t s);
xk_status xk_exclusive_scan_i64(const int64_t* in, int64_t* out, long long n, int64_t* total_dev,
                                cudaStream_t s);
// Number of block sums the scans use for n elements, and the int32 scan with a
// caller-provided block-sum array of bsum_cap words (same kernels, same result;
// allocates nothing).
long long xk_scan_tiles(long long n);
xk_status xk_exclusive_scan_i32_scratch(const int32_t* in, int32_t* out, long long n, int64_t* total_dev,
                                        int64_t* bsum, long long bsum_cap, cudaStream_t s);
// Stable LSD radix sort of 64-bit keys with 32-bit values; `bits` low key bits are sorted.
xk_status xk_radix_sort_u64(uint64_t* keys, int32_t* vals, long long n, int bits, cudaStream_t s);
