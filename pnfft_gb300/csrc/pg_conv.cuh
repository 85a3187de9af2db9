// pg_conv.cuh -- device helpers shared by the convolution kernels (conv.cu,
// interp_group.cu, interp_tile.cuh, spread_line.cuh, generic.cu): the
// node -> grid index, complex types, warp reduction, tile geometry, window
// values of one stencil point, and the node records of the binning.
#pragma once
#include <cuda_runtime.h>

#include "pg_kernels.h"
#include "pg_math.cuh"

namespace pg {

// ---------------------------------------------------------------------------
// node -> grid index, bit-exact with ndft-parallel.c:2732-2753, 2165-2174:
// x' = x (+ 0.5/n when interlaced), fnx = floor(n x'), u = fnx - m, then the
// fold x' -= 1 (fnx -= n) when x' >= 0.5.  Explicit _rn intrinsics keep nvcc
// from fusing the operations into an FMA.
// ---------------------------------------------------------------------------
struct AxisPos {
  double dist;  // n x' - fnx after the fold, in [0,1)
  int u;        // lowest stencil index wrapped into [0, n)
};

__device__ __forceinline__ AxisPos axis_pos(double x, int n, int m, int il) {
  double xs = x;
  if (il) xs = __dadd_rn(xs, __ddiv_rn(0.5, (double)n));
  double fnx = floor(__dmul_rn((double)n, xs));
  long long u = (long long)fnx - m;
  if (il && xs >= 0.5) {
    xs = __dsub_rn(xs, 1.0);
    fnx -= (double)n;
  }
  AxisPos p;
  p.dist = __dsub_rn(__dmul_rn((double)n, xs), fnx);
  long long w = u % n;
  if (w < 0) w += n;
  p.u = (int)w;
  return p;
}

template <typename T>
struct Cplx;
template <>
struct Cplx<float> {
  typedef float2 type;
};
template <>
struct Cplx<double> {
  typedef double2 type;
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void tile_base(const Binning &b, int tile, int *base) {
  int t2 = tile % b.ntile[2];
  int r = tile / b.ntile[2];
  int t1 = r % b.ntile[1];
  int t0 = r / b.ntile[1];
  base[0] = t0 * b.T[0];
  base[1] = t1 * b.T[1];
  base[2] = t2 * b.T[2];
}

// acc += w * g for a complex g and a real weight w: the paired FMA of sm_100+
// in FP32 (each component rounds like fmaf), two FMAs in FP64
__device__ __forceinline__ void cfma(float2 &acc, float w, float2 g) { acc = __ffma2_rn(make_float2(w, w), g, acc); }
__device__ __forceinline__ void cfma(double2 &acc, double w, double2 g) {
  acc.x = fma(w, g.x, acc.x);
  acc.y = fma(w, g.y, acc.y);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// copies the R^3 region of the grid starting at base (wrapped modulo n) into
// shared memory, row-major with z fastest; R even.  FP32 grids with even n2
// move two complex values per 16-byte load (pairs never straddle the wrap:
// base2 and n2 are even).
template <int R, typename C>
__device__ __forceinline__ void load_region(C *reg, const C *__restrict__ grid, const int *base, int n0, int n1,
                                            int n2, int real_only) {
  static_assert(R % 2 == 0, "region rows hold pairs");
  if (sizeof(C) == 8 && (n2 & 1) == 0) {
    constexpr int RP = R / 2;
#pragma unroll 4
    for (int i = threadIdx.x; i < R * R * RP; i += blockDim.x) {
      const int cp = i % RP, q = i / RP;
      const int bb = q % R, aa = q / R;
      int g0 = base[0] + aa, g1 = base[1] + bb, g2 = base[2] + 2 * cp;
      if (g0 >= n0) g0 %= n0;
      if (g1 >= n1) g1 %= n1;
      if (g2 >= n2) g2 %= n2;
      float4 v = *(const float4 *)(grid + ((size_t)g0 * n1 + g1) * n2 + g2);
      if (real_only) v.y = v.w = 0.f;
      *(float4 *)(reg + (aa * R + bb) * R + 2 * cp) = v;
    }
    return;
  }
  for (int i = threadIdx.x; i < R * R * R; i += blockDim.x) {
    const int c = i % R, q = i / R;
    const int bb = q % R, aa = q / R;
    int g0 = base[0] + aa, g1 = base[1] + bb, g2 = base[2] + c;
    if (g0 >= n0) g0 %= n0;
    if (g1 >= n1) g1 %= n1;
    if (g2 >= n2) g2 %= n2;
    C v = grid[((size_t)g0 * n1 + g1) * n2 + g2];
    if (real_only) v.y = 0;
    reg[i] = v;
  }
}

__device__ __forceinline__ void atomic_add_grid(float2 *p, float2 v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_grid(double2 *p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

// ---------------------------------------------------------------------------
// shared helpers of the tiled kernels (8x8x8-cell tiles, compile-time cutoff)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void window_formula(const WindowArgs &w, int t, int s, float dist, int nder, float *out) {
  window_eval_f(w.kind, w.m, w.wf[t], w.m - s, dist, nder, out);
}
__device__ __forceinline__ void window_formula(const WindowArgs &w, int t, int s, double dist, int nder,
                                               double *out) {
  window_eval<double>(w.kind, w.m, (double)w.n[t], w.b[t], dist + (double)(w.m - s), (double)s - dist, nder, out);
}

// FP32: Horner on the fitted polynomial of stencil point s (16 or 12 FMAs per value)
__device__ __forceinline__ float poly_horner(const float4 &c0, const float4 &c1, const float4 &c2, const float4 &c3,
                                             float u) {
  float h = c3.w;
  h = fmaf(h, u, c3.z);
  h = fmaf(h, u, c3.y);
  h = fmaf(h, u, c3.x);
  h = fmaf(h, u, c2.w);
  h = fmaf(h, u, c2.z);
  h = fmaf(h, u, c2.y);
  h = fmaf(h, u, c2.x);
  h = fmaf(h, u, c1.w);
  h = fmaf(h, u, c1.z);
  h = fmaf(h, u, c1.y);
  h = fmaf(h, u, c1.x);
  h = fmaf(h, u, c0.w);
  h = fmaf(h, u, c0.z);
  h = fmaf(h, u, c0.y);
  return fmaf(h, u, c0.x);
}
// the same with the top four coefficients zero: Horner from a zero leading
// term reaches c2.w exactly, so both give the same bits for such rows
__device__ __forceinline__ float poly_horner12(const float4 &c0, const float4 &c1, const float4 &c2, float u) {
  float h = c2.w;
  h = fmaf(h, u, c2.z);
  h = fmaf(h, u, c2.y);
  h = fmaf(h, u, c2.x);
  h = fmaf(h, u, c1.w);
  h = fmaf(h, u, c1.z);
  h = fmaf(h, u, c1.y);
  h = fmaf(h, u, c1.x);
  h = fmaf(h, u, c0.w);
  h = fmaf(h, u, c0.z);
  h = fmaf(h, u, c0.y);
  return fmaf(h, u, c0.x);
}
__device__ __forceinline__ float poly_eval(const float *row, float u, int ncoef) {
  const float4 *r = (const float4 *)row;
  if (ncoef <= 12) return poly_horner12(__ldg(r), __ldg(r + 1), __ldg(r + 2), u);
  return poly_horner(__ldg(r), __ldg(r + 1), __ldg(r + 2), __ldg(r + 3), u);
}

// psi (and derivatives up to nder) of stencil points 2 cp and 2 cp + 1 on
// axis t from the paired polynomial rows (FP32-mixed plans with fitted
// polynomials), two points per paired FMA: each lane rounds like fmaf, in the
// Horner order of poly_eval, so the values equal window_point's bit for bit
// (except the Bessel-I0 point that window_point evaluates by the formula)
__device__ __forceinline__ void window_pair(const WindowArgs &w, int t, int cp, float dist, int nder, float2 *out) {
  const int np = (w.cut + 1) / 2;
  const float u = dist - 0.5f;
  const float2 u2 = make_float2(u, u);
  for (int d = 0; d <= nder; d++) {
    const float4 *r = (const float4 *)(w.poly_pp + ((d * 3 + t) * np + cp) * 32);  // r[j]: coefficients 2j, 2j + 1
    float2 h;
    if (w.poly_ncoef <= 12) {
      const float4 q5 = __ldg(r + 5);
      h = make_float2(q5.z, q5.w);
      h = __ffma2_rn(h, u2, make_float2(q5.x, q5.y));
    } else {
      const float4 q7 = __ldg(r + 7), q6 = __ldg(r + 6), q5 = __ldg(r + 5);
      h = make_float2(q7.z, q7.w);
      h = __ffma2_rn(h, u2, make_float2(q7.x, q7.y));
      h = __ffma2_rn(h, u2, make_float2(q6.z, q6.w));
      h = __ffma2_rn(h, u2, make_float2(q6.x, q6.y));
      h = __ffma2_rn(h, u2, make_float2(q5.z, q5.w));
      h = __ffma2_rn(h, u2, make_float2(q5.x, q5.y));
    }
#pragma unroll
    for (int j = 4; j >= 0; j--) {
      const float4 q = __ldg(r + j);
      h = __ffma2_rn(h, u2, make_float2(q.z, q.w));
      h = __ffma2_rn(h, u2, make_float2(q.x, q.y));
    }
    out[d] = h;
  }
}

// psi (and derivatives up to nder) of stencil point s on axis t for a node at
// fractional position dist, from the interpolation table, the fitted
// polynomial (FP32) or the formula
template <typename T>
__device__ __forceinline__ void window_point(const WindowArgs &w, int t, int s, T dist, int nder, T *out) {
  if constexpr (sizeof(T) == 4) {
    // the Bessel-I0 window jumps from 1/2 to 0 at y = m (s = 0, dist = 0)
    if (w.poly && w.intpol_order < 0 && !(w.kind == WIN_BESSEL_I0 && s == 0 && dist == 0.f)) {
      const float u = dist - 0.5f;
      for (int d = 0; d <= nder; d++)
        out[d] = poly_eval(w.poly + ((d * 3 + t) * w.cut + s) * kPolyCoef, u, w.poly_ncoef);
      return;
    }
  }
  if (w.intpol_order >= 0) {
    // an FP32 fraction can round up to exactly 1 (FP64 ones stay below 1):
    // the last sub-interval, evaluated at its right end, gives the window there
    T dK = dist * (T)w.intpol_K;
    int k = min((int)floor(dK), w.intpol_K - 1);
    T dk = dK - (T)k;
    size_t base = ((size_t)k * w.cut + s) * (size_t)(w.intpol_order + 1);
    for (int d = 0; d <= nder; d++) out[d] = intpol<T>(w.intpol_order, (const T *)w.tab[d][t] + base, dk);
  } else {
    window_formula(w, t, s, dist, nder, out);
  }
}

__device__ __forceinline__ void unpack_corner(int pk, int *o) {
  o[0] = pk & 0xff;
  o[1] = (pk >> 8) & 0xff;
  o[2] = (pk >> 16) & 0xff;
}

__device__ __forceinline__ void load_rec_raw(const void *rec, int pos, float *d, int *pk) {
  float4 r = ((const float4 *)rec)[pos];
  d[0] = r.x;
  d[1] = r.y;
  d[2] = r.z;
  *pk = __float_as_int(r.w);
}
__device__ __forceinline__ void load_rec_raw(const void *rec, int pos, double *d, int *pk) {
  double4 r = ((const double4 *)rec)[pos];
  d[0] = r.x;
  d[1] = r.y;
  d[2] = r.z;
  *pk = (int)__double_as_longlong(r.w);
}

}  // namespace pg
