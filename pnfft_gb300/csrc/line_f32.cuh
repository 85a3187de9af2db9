// line_f32.cuh -- shared pieces of the FP32-mixed line kernels of f alone:
// the interpolation B (interp_line.cu) and the spreading B^T
// (spread_line_f.cu).  One CTA takes the nodes of one line of 4x4x4-cell
// tiles along axis 2 (sorted by slab = u2 / 4); thread (a, b) owns the grid
// columns (a, b) and (a, b + R/2) of the line's (3+CUT)^2 region and keeps W
// consecutive z values of each in registers, in rotation: slot p holds the
// z of the window with z = p (mod W), and the window of slab s covers z in
// [4s, 4s + W).  A node's z row is staged in the same rotation, so every
// column update or z sum is one branch-free run over the W slots.
#pragma once
#include <cuda_runtime.h>

#include "pg_conv.cuh"
#include "pg_kernels.h"
#include "pg_math.cuh"

namespace pg {

template <int CUT>
struct LineGeom32 {
  static constexpr int TL = 4;                   // tile edge in every axis
  static constexpr int R = TL + CUT - 1;         // region edge in axes 0, 1
  static constexpr int HR = R / 2;               // column pairs per region row
  static constexpr int W = (CUT + TL - 1 <= 8) ? 8 : 16;  // z slots (power of two)
  static constexpr int NG = W / 4;               // groups of 4 slots
  static constexpr int THREADS = (R * HR + 31) / 32 * 32;
  static constexpr int NB = THREADS / 4;         // nodes per batch: 4 threads reduce each
  static constexpr int WS = W + 32 + 4;          // floats per node row (z slots, x rows, y pairs, pad)
  static constexpr int PS = 20;                  // shared-memory stride of a polynomial row (16 used)
  static constexpr int PR = THREADS + 4;         // float2 per node row of the shares
  static_assert(R % 2 == 0 && R <= 16, "region rows and column pairs fit the staged rows");
  static_assert(CUT + TL - 1 <= W, "a slab's stencils fit the z window");
  static_assert(WS % 4 == 0, "16-byte aligned node rows");
};

__device__ __forceinline__ int wrap_n(int z, int n) {
  if (z >= n) z -= n;
  if (z >= n) z %= n;
  return z;
}

// loads the 4 z values z0 .. z0+3 (wrapped) of a grid column into v[0..3]
__device__ __forceinline__ void load_z4(const float2 *__restrict__ col, int z0, int n2, bool vec, int real_only,
                                        float2 *v) {
  if (vec) {  // n2 % 4 == 0: z0 wraps to a multiple of 4, the 4 values are contiguous and 32-byte aligned
    const float4 *p = (const float4 *)(col + wrap_n(z0, n2));
    const float4 a = __ldg(p), b = __ldg(p + 1);
    v[0] = make_float2(a.x, a.y);
    v[1] = make_float2(a.z, a.w);
    v[2] = make_float2(b.x, b.y);
    v[3] = make_float2(b.z, b.w);
  } else {
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = __ldg(col + wrap_n(z0 + k, n2));
  }
  if (real_only) {
#pragma unroll
    for (int k = 0; k < 4; k++) v[k].y = 0.f;
  }
}

// asynchronous 16-byte copy global -> shared (completion per thread: the
// thread that issued it waits and reads it)
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// the psi row of one node on one axis: CUT values from the fitted polynomial
// rows in shared memory (the same rows for a whole warp) or the generic window
template <int CUT>
__device__ __forceinline__ void window_row(const WindowArgs &w, bool poly, const float *s_poly, int t, float dist,
                                           float *v) {
  constexpr int PS = LineGeom32<CUT>::PS;
#pragma unroll
  for (int c = 0; c < CUT; c++) {
    if (poly && !(w.kind == WIN_BESSEL_I0 && c == 0 && dist == 0.f)) {
      const float4 *rw = (const float4 *)(s_poly + (t * CUT + c) * PS);
      v[c] = w.poly_ncoef <= 12 ? poly_horner12(rw[0], rw[1], rw[2], dist - 0.5f)
                                : poly_horner(rw[0], rw[1], rw[2], rw[3], dist - 0.5f);
    } else {
      float out[3];
      window_point<float>(w, t, c, dist, 0, out);
      v[c] = out[0];
    }
  }
}

// The FP32 window polynomials in pairs of stencil points, for paired FMAs:
// for polynomial row r (derivative der and axis t: r = 3 der + t) and pair
// cp (points 2 cp and 2 cp + 1), coefficient k of both points at
// s_pp[((r * NP + cp) * 16 + k) * 2 + {0, 1}] (zero for a point beyond CUT),
// so that one 16-byte load gives two coefficients of the pair.
template <int CUT, int NROWS = 3>
struct PolyPairs {
  static constexpr int NP = (CUT + 1) / 2;
  static constexpr int FLOATS = NROWS * NP * 32;
};

template <int CUT, int NTH, int NROWS = 3>
__device__ __forceinline__ void stage_poly_pairs(const float *poly, float *s_pp, int tid) {
  constexpr int NP = PolyPairs<CUT>::NP;
  for (int i = tid; i < NROWS * NP * 16; i += NTH) {
    const int k = i & 15, cp = (i >> 4) % NP, r = (i >> 4) / NP;
    const int c0 = 2 * cp, c1 = c0 + 1;
    const float v0 = __ldg(poly + (r * CUT + c0) * kPolyCoef + k);
    const float v1 = c1 < CUT ? __ldg(poly + (r * CUT + c1) * kPolyCoef + k) : 0.f;
    *(float2 *)(s_pp + 2 * i) = make_float2(v0, v1);
  }
}

// Derivative `der` of the window row of one node on axis t (CUT values) as
// the single-row evaluation, two stencil points per paired FMA: each lane
// rounds like fmaf, in the same Horner order, so the values are the same bit
// for bit
template <int CUT>
__device__ __forceinline__ void window_row_pp_d(const WindowArgs &w, bool poly, const float *s_pp, int der, int t,
                                                float dist, float *v) {
  constexpr int NP = PolyPairs<CUT>::NP;
  if (!poly) {
#pragma unroll
    for (int c = 0; c < CUT; c++) {
      float out[3];
      window_point<float>(w, t, c, dist, der, out);
      v[c] = out[der];
    }
    return;
  }
  const float u = dist - 0.5f;
  const float2 u2 = make_float2(u, u);
  const bool short_rows = w.poly_ncoef <= 12;
  const int row = 3 * der + t;
#pragma unroll
  for (int cp = 0; cp < NP; cp++) {
    const float4 *r = (const float4 *)(s_pp + (row * NP + cp) * 32);  // r[j]: coefficients 2j, 2j + 1 of both points
    float2 h;
    if (short_rows) {
      const float4 q5 = r[5];
      h = make_float2(q5.z, q5.w);
      h = __ffma2_rn(h, u2, make_float2(q5.x, q5.y));
    } else {
      const float4 q7 = r[7], q6 = r[6], q5 = r[5];
      h = make_float2(q7.z, q7.w);
      h = __ffma2_rn(h, u2, make_float2(q7.x, q7.y));
      h = __ffma2_rn(h, u2, make_float2(q6.z, q6.w));
      h = __ffma2_rn(h, u2, make_float2(q6.x, q6.y));
      h = __ffma2_rn(h, u2, make_float2(q5.z, q5.w));
      h = __ffma2_rn(h, u2, make_float2(q5.x, q5.y));
    }
#pragma unroll
    for (int j = 4; j >= 0; j--) {
      const float4 q = r[j];
      h = __ffma2_rn(h, u2, make_float2(q.z, q.w));
      h = __ffma2_rn(h, u2, make_float2(q.x, q.y));
    }
    v[2 * cp] = h.x;
    if (2 * cp + 1 < CUT) v[2 * cp + 1] = h.y;
  }
  if (w.kind == WIN_BESSEL_I0 && dist == 0.f) {  // the fit is not used at the removable singularity
    float out[3];
    window_point<float>(w, t, 0, dist, der, out);
    v[0] = out[der];
  }
}

template <int CUT>
__device__ __forceinline__ void window_row_pp(const WindowArgs &w, bool poly, const float *s_pp, int t, float dist,
                                              float *v) {
  window_row_pp_d<CUT>(w, poly, s_pp, 0, t, dist, v);
}

// Kahan-compensated sum of the shares part[r], part[r + 4], ... (below NTH)
// in a fixed order, returned as the compensated value (sum minus the carried
// correction).  The four threads r = 0..3 of a node each take a
// quarter of the node's shares: a plain FP32 run of NTH / 4 additions is the
// largest rounding term of the interpolation (about two thirds of the FP32
// error of B on uniform nodes at m = 6), compensation leaves it at the level
// of the grid and window rounding.
template <int NTH>
__device__ __forceinline__ float2 kahan_quarter_sum(const float2 *part, int r) {
  // two compensated runs (shares r, r + 8, ... and r + 4, r + 12, ...) halve
  // the length of the dependent chain
  float2 s = make_float2(0.f, 0.f), c = s, u = s, e = s;
#pragma unroll 4
  for (int k = r; k < NTH; k += 8) {
    const float2 y = __fadd2_rn(part[k], make_float2(-c.x, -c.y));
    const float2 t = __fadd2_rn(s, y);
    c = __fadd2_rn(__fadd2_rn(t, make_float2(-s.x, -s.y)), make_float2(-y.x, -y.y));
    s = t;
    const float2 y2 = __fadd2_rn(part[k + 4], make_float2(-e.x, -e.y));
    const float2 t2 = __fadd2_rn(u, y2);
    e = __fadd2_rn(__fadd2_rn(t2, make_float2(-u.x, -u.y)), make_float2(-y2.x, -y2.y));
    u = t2;
  }
  // s + u with its rounding error (TwoSum), then the two corrections
  const float2 t = __fadd2_rn(s, u);
  const float2 bb = __fadd2_rn(t, make_float2(-s.x, -s.y));
  const float2 err = __fadd2_rn(__fadd2_rn(s, make_float2(-(t.x - bb.x), -(t.y - bb.y))),
                                __fadd2_rn(u, make_float2(-bb.x, -bb.y)));
  return __fadd2_rn(t, __fadd2_rn(err, make_float2(-(c.x + e.x), -(c.y + e.y))));
}

// The item and sub-problem of block `blk` of a MultiConv launch, and a copy of
// the item's arguments in shared memory (all threads of the block).
__device__ __forceinline__ int multi_item(const MultiConv &mc, int blk) {
  int lo = 0, hi = mc.n - 1;  // the last item with first[item] <= blk
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mc.first[mid] <= blk) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void copy_args(ConvArgs *dst, const ConvArgs *src) {
  static_assert(sizeof(ConvArgs) % 8 == 0, "ConvArgs copied in 8-byte words");
  const unsigned long long *s = (const unsigned long long *)src;
  unsigned long long *d = (unsigned long long *)dst;
  for (int i = threadIdx.x; i < (int)(sizeof(ConvArgs) / 8); i += blockDim.x) d[i] = s[i];
  __syncthreads();
}

}  // namespace pg
