// interp_line.cu -- interpolation B of the FP32-mixed plans (f only) along
// lines of tiles: the transpose of the spreading of spread_line.cuh, on the
// same binning.
//
// Reference: loop_over_particles_trafo (kernel/ndft-parallel.c:2703-2888)
// with the interpolation loops of kernel/assign.c:667-691.
#include <cuda_runtime.h>

#include "pg_conv.cuh"
#include "pg_kernels.h"
#include "pg_math.cuh"

namespace pg {

// ---------------------------------------------------------------------------
// One CTA takes the nodes of one line of 4x4x4-cell tiles running along axis
// 2 (sorted by slab = u2 / 4), or a run of at most sub_max of them.  The
// (3+CUT)^2 region of the line in axes 0, 1 is split into column pairs:
// thread (a, b) owns the grid columns (a, b) and (a, b + R/2) and keeps W
// consecutive z values of each in registers: slot p holds the value at the
// z of the window with z = p (mod W), and the window of slab s covers z in
// [4s, 4s + W).  Moving to a later slab replaces whole groups of 4 slots
// (loads only, no register moves), and the node's z window row is staged in
// the same rotation, so the z sum of a column is a branch-free W-long FMA run:
//   s_c = sum_p psi_z'[p] g_c[p]         (psi_z' zero outside the stencil)
// The thread's share of the node's value is psi_x[a] (psi_y[b] s_0 +
// psi_y[b + R/2] s_1); the shares of all threads are added in a fixed order
// in shared memory (four threads per node, then two shuffles), so a node's
// result depends only on the node.
// Window values are evaluated stencil-point-major (a warp takes one stencil
// point of one axis for 32 nodes, so the fitted polynomial's coefficients
// are broadcast reads) into zeroed rows: the node's z row in slot rotation,
// its x row over the region's rows and its y row over the region's column
// pairs.
// ---------------------------------------------------------------------------
template <int CUT>
struct ILGeom {
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

template <int CUT>
__global__ void __launch_bounds__(ILGeom<CUT>::THREADS, 4) k_interp_line(ConvArgs a) {
  typedef ILGeom<CUT> G;
  constexpr int TL = G::TL, R = G::R, HR = G::HR, W = G::W, NG = G::NG, NB = G::NB, WS = G::WS, PS = G::PS,
                PR = G::PR, NTH = G::THREADS;
  __shared__ __align__(16) float s_w[NB][WS];
  __shared__ __align__(16) float2 s_part[NB][PR];
  __shared__ __align__(16) float s_poly[3 * CUT * PS];
  __shared__ float s_d[NB][3];
  __shared__ int s_o[NB], s_j[NB];
  const Binning &b = a.bin;
  const int sub = blockIdx.x;
  if (sub >= *b.nsub) return;
  const int line = b.sub_tile[sub], first = b.sub_first[sub], cnt = b.sub_cnt[sub];
  if (cnt <= 0) return;  // a line without nodes
  const int t1 = line % b.ntile[1], t0 = line / b.ntile[1];
  const int tid = threadIdx.x;
  const bool active = tid < R * HR;
  const int ca = active ? tid / HR : 0, cb = active ? tid % HR : 0;
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  const size_t gx = (size_t)((t0 * TL + ca) % n0) * n1;
  const float2 *grid = (const float2 *)a.grid;
  const float2 *col0 = grid + (gx + (t1 * TL + cb) % n1) * n2;
  const float2 *col1 = grid + (gx + (t1 * TL + cb + HR) % n1) * n2;
  const bool vec = (n2 & 3) == 0;
  const WindowArgs &w = a.w;
  const bool poly = w.poly && w.intpol_order < 0;
  if (poly)
    for (int i = tid; i < 3 * CUT * 4; i += NTH)
      ((float4 *)(s_poly + (i >> 2) * PS))[i & 3] = __ldg((const float4 *)(w.poly + (i >> 2) * kPolyCoef) + (i & 3));
  const float scale = a.use_il ? 0.5f : 1.f;

  float2 g0[W], g1[W];  // the two columns' z windows, slot p holds z = p (mod W)
#pragma unroll
  for (int p = 0; p < W; p++) g0[p] = g1[p] = make_float2(0.f, 0.f);
  int zs = -1;  // slab of the window (-1: none loaded)

  for (int b0 = 0; b0 < cnt; b0 += NB) {
    const int nb = min(NB, cnt - b0);
    __syncthreads();  // the previous batch's rows and shares are consumed
    // --- stage the node records and clear the window rows ---------------------
    if (tid < nb) {
      const float4 r = ((const float4 *)b.rec)[first + b0 + tid];
      s_d[tid][0] = r.x;
      s_d[tid][1] = r.y;
      s_d[tid][2] = r.z;
      s_o[tid] = __float_as_int(r.w);
      s_j[tid] = b.perm[first + b0 + tid];
    }
    for (int v = tid; v < nb * (WS / 4); v += NTH) ((float4 *)&s_w[0][0])[v] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    // --- window values, stencil-point-major -------------------------------------
    for (int v = tid; v < 3 * CUT * NB; v += NTH) {
      const int e = v / NB, i = v - e * NB;
      if (i >= nb) continue;
      const int t = e / CUT, c = e - t * CUT;
      const float dist = s_d[i][t];
      float val;
      if (poly && !(w.kind == WIN_BESSEL_I0 && c == 0 && dist == 0.f)) {
        const float4 *rw = (const float4 *)(s_poly + e * PS);
        val = w.poly_ncoef <= 12 ? poly_horner12(rw[0], rw[1], rw[2], dist - 0.5f)
                                 : poly_horner(rw[0], rw[1], rw[2], rw[3], dist - 0.5f);
      } else {
        float out[3];
        window_point<float>(w, t, c, dist, 0, out);
        val = out[0];
      }
      const int pk = s_o[i];
      int pos;
      if (t == 2) {
        pos = (((pk >> 16) & 0x7fff) + c) & (W - 1);  // z slot
      } else if (t == 0) {
        pos = W + (pk & 0xff) + c;  // region row
      } else {
        const int bc = ((pk >> 8) & 0xff) + c;  // region column -> (pair, element)
        pos = W + 16 + 2 * (bc % HR) + bc / HR;
      }
      s_w[i][pos] = val;
    }
    __syncthreads();
    // --- the z sums of the thread's two columns, node by node --------------------
    for (int i = 0; i < nb; i++) {
      const int slab = ((s_o[i] >> 16) & 0x7fff) >> 2;
      if (slab != zs) {
        // group q of the new window holds z = 4 (slab + ((q - slab) mod NG)); it
        // is loaded unless the old window already holds it
#pragma unroll
        for (int q = 0; q < NG; q++) {
          const int zq = 4 * (slab + ((q - slab) & (NG - 1)));
          if (zs < 0 || zq >= 4 * zs + W) {
            if (active) {
              load_z4(col0, zq, n2, vec, a.real_only, &g0[4 * q]);
              load_z4(col1, zq, n2, vec, a.real_only, &g1[4 * q]);
            }
          }
        }
        zs = slab;
      }
      const float4 *pz4 = (const float4 *)s_w[i];
      float2 s0a = make_float2(0.f, 0.f), s0b = s0a, s1a = s0a, s1b = s0a;
#pragma unroll
      for (int q = 0; q < NG; q++) {
        const float4 z = pz4[q];
        s0a = __ffma2_rn(g0[4 * q], make_float2(z.x, z.x), s0a);
        s1a = __ffma2_rn(g1[4 * q], make_float2(z.x, z.x), s1a);
        s0b = __ffma2_rn(g0[4 * q + 1], make_float2(z.y, z.y), s0b);
        s1b = __ffma2_rn(g1[4 * q + 1], make_float2(z.y, z.y), s1b);
        s0a = __ffma2_rn(g0[4 * q + 2], make_float2(z.z, z.z), s0a);
        s1a = __ffma2_rn(g1[4 * q + 2], make_float2(z.z, z.z), s1a);
        s0b = __ffma2_rn(g0[4 * q + 3], make_float2(z.w, z.w), s0b);
        s1b = __ffma2_rn(g1[4 * q + 3], make_float2(z.w, z.w), s1b);
      }
      const float px = s_w[i][W + ca];
      const float2 py = ((const float2 *)(s_w[i] + W + 16))[cb];
      const float2 s0 = __fadd2_rn(s0a, s0b), s1 = __fadd2_rn(s1a, s1b);
      float2 t = __fmul2_rn(s0, make_float2(py.x, py.x));
      t = __ffma2_rn(s1, make_float2(py.y, py.y), t);
      t = __fmul2_rn(t, make_float2(px, px));
      s_part[i][tid] = active ? t : make_float2(0.f, 0.f);
    }
    __syncthreads();
    // --- the node sums: four threads per node, a fixed order -----------------------
    {
      const int i = tid >> 2, r = tid & 3;
      float2 s = make_float2(0.f, 0.f);
      if (i < nb) {
#pragma unroll 8
        for (int k = r; k < NTH; k += 4) s = __fadd2_rn(s, s_part[i][k]);
      }
      s.x += __shfl_xor_sync(0xffffffffu, s.x, 1);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, 1);
      s.x += __shfl_xor_sync(0xffffffffu, s.x, 2);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, 2);
      if (i < nb && r == 0) {
        const int64_t e = (int64_t)s_j[i] * a.stride + a.offset;
        const double vr = (double)(s.x * scale), vi = (double)(s.y * scale);
        if (a.real_io) {
          if (a.accum) a.f_out[e] += vr;
          else a.f_out[e] = vr;
        } else {
          double2 *o2 = (double2 *)a.f_out + e;
          if (a.accum) {
            double2 o = *o2;
            o.x += vr;
            o.y += vi;
            *o2 = o;
          } else {
            *o2 = make_double2(vr, vi);
          }
        }
      }
    }
  }
}

template <int CUT>
static void run_interp_line(const ConvArgs &a, cudaStream_t s) {
  k_interp_line<CUT><<<a.bin.max_subs, ILGeom<CUT>::THREADS, 0, s>>>(a);
}

bool launch_interp_line(const ConvArgs &a, cudaStream_t s) {
  switch (a.w.cut) {
    case 5: run_interp_line<5>(a, s); return true;
    case 7: run_interp_line<7>(a, s); return true;
    case 9: run_interp_line<9>(a, s); return true;
    case 11: run_interp_line<11>(a, s); return true;
    case 13: run_interp_line<13>(a, s); return true;
    default: return false;
  }
}

}  // namespace pg
