// Layered helical strand meshes generated on the device: the geometry of the
// reference's twisted-wire generator (xkep_cae/mesh/_twisted_wire.py:150-383)
// for many strands at once, so that the batched many-strand workload is built
// where it is assembled.  Wire 0 is a straight core; layer k holds 6k wire
// slots at angles 2 pi j / 6k on a helix of lay radius k (d + gap); odd layers
// twist in lay_direction, even layers the other way; a three-wire strand has
// no core (three wires at (d + gap) / sqrt(3)).  Node positions follow the
// generator's arithmetic: the core's z is numpy's linspace (i * step, the last
// point pinned to the length), a helix's z is (i * length) / (n - 1) and its
// angle ((dir * 2) * pi) * z / pitch + offset, each operation rounded on its
// own.  Positions can differ from the host's libm by the last bit of cos / sin.
#include <math.h>

#include "xk_common.cuh"

namespace {

constexpr double XK_PI = 3.141592653589793;

struct WirePlace {
  int layer;
  double angle, radius;
  int direction;
};

XK_D WirePlace wire_place(const xk_strand_spec& sp, int w) {
  WirePlace p;
  const double d_gap = xadd(sp.wire_diameter, sp.gap);
  if (sp.n_wires == 3) {
    p.layer = 1;
    p.angle = xdiv(xmul(xmul(2.0, XK_PI), (double)w), 3.0);
    p.radius = xdiv(d_gap, sqrt(3.0));
    p.direction = sp.lay_direction;
    return p;
  }
  if (w == 0) {
    p.layer = 0;
    p.angle = 0.0;
    p.radius = 0.0;
    p.direction = 0;
    return p;
  }
  int k = 1, first = 1;  // first wire of layer k: 1 + 3k(k-1)
  while (w >= first + 6 * k) {
    first += 6 * k;
    ++k;
  }
  p.layer = k;
  p.angle = xdiv(xmul(xmul(2.0, XK_PI), (double)(w - first)), (double)(6 * k));
  p.radius = xmul((double)k, d_gap);
  p.direction = (k % 2 == 1) ? sp.lay_direction : -sp.lay_direction;
  return p;
}

// index of the spec whose range [first, next first) holds item v (specs sorted by first)
template <bool NODES>
XK_D int find_spec(const xk_strand_spec* __restrict__ sp, int n, long long v) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const long long f = NODES ? sp[mid].node_first : sp[mid].elem_first;
    if (f <= v) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void k_strand_nodes(const xk_strand_spec* __restrict__ specs, int n_specs, long long n_nodes,
                               double* __restrict__ X) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_nodes) return;
  const xk_strand_spec sp = specs[find_spec<true>(specs, n_specs, v)];
  const int npw = sp.n_elems_per_wire + 1;
  const long long local = v - sp.node_first;
  const int w = (int)(local / npw), i = (int)(local % npw);
  const WirePlace p = wire_place(sp, w);
  double x, y, z;
  if (p.radius < 1e-15) {  // straight core: numpy linspace(0, length, npw)
    const double step = xdiv(sp.length, (double)(npw - 1));
    z = (i == npw - 1) ? sp.length : xadd(xmul((double)i, step), 0.0);
    x = 0.0;
    y = 0.0;
  } else {
    z = xdiv(xmul((double)i, sp.length), (double)(npw - 1));
    const double th = xadd(xdiv(xmul(xmul(xmul((double)p.direction, 2.0), XK_PI), z), sp.pitch), p.angle);
    x = xmul(p.radius, cos(th));
    y = xmul(p.radius, sin(th));
  }
  X[3 * v] = xadd(x, sp.x_offset);
  X[3 * v + 1] = y;
  X[3 * v + 2] = z;
}

__global__ void k_strand_elems(const xk_strand_spec* __restrict__ specs, int n_specs, long long n_elems,
                               int32_t* __restrict__ conn, int32_t* __restrict__ layer, double* __restrict__ radii) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  const xk_strand_spec sp = specs[find_spec<false>(specs, n_specs, e)];
  const long long local = e - sp.elem_first;
  const int w = (int)(local / sp.n_elems_per_wire), i = (int)(local % sp.n_elems_per_wire);
  const long long n0 = sp.node_first + (long long)w * (sp.n_elems_per_wire + 1) + i;
  conn[2 * e] = (int32_t)n0;
  conn[2 * e + 1] = (int32_t)(n0 + 1);
  if (layer) layer[e] = wire_place(sp, w).layer;
  if (radii) radii[e] = xmul(sp.wire_diameter, 0.5);
}

}  // namespace

extern "C" xk_status xk_strand_generate(const xk_strand_spec* specs, int32_t n_specs, int64_t n_nodes,
                                        int64_t n_elems, double* X, int32_t* conn, int32_t* elem_layer,
                                        double* radii, xk_stream s) {
  if (!specs || n_specs <= 0 || n_nodes < 0 || n_elems < 0 || (n_nodes > 0 && !X) || (n_elems > 0 && !conn))
    return xk_set_error(XK_ERR_ARG, "xk_strand_generate: bad arguments");
  if (n_nodes > 0x7fffffffLL) return xk_set_error(XK_ERR_ARG, "xk_strand_generate: node ids must fit int32");
  cudaStream_t st = (cudaStream_t)s;
  if (n_nodes > 0) k_strand_nodes<<<xk_blocks(n_nodes, 256), 256, 0, st>>>(specs, n_specs, n_nodes, X);
  if (n_elems > 0)
    k_strand_elems<<<xk_blocks(n_elems, 256), 256, 0, st>>>(specs, n_specs, n_elems, conn, elem_layer, radii);
  XK_CHECK_LAUNCH();
  return XK_OK;
}
