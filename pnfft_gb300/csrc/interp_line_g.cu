// interp_line_g.cu -- interpolation B of the FP32-mixed plans with the
// gradient (COMPUTE_GRAD_F, with or without COMPUTE_F) along lines of tiles,
// on the line binning that the spreading and k_interp_line use.
//
// Reference: loop_over_particles_trafo (kernel/ndft-parallel.c:2703-2888)
// with the gradient loops of kernel/assign.c:763-793 and 1033-1066.
#include <cuda_runtime.h>

#include "line_f32.cuh"

namespace pg {

// ---------------------------------------------------------------------------
// Geometry and the rotating z window as in line_f32.cuh and k_interp_line.
// Per node each thread forms, for its two grid columns, the z sums with the
// window and with its derivative,
//   s_c = sum_p psi_z'[p] g_c[p],   t_c = sum_p dpsi_z'[p] g_c[p],
// and from them its shares of
//   f   = psi_x  (psi_y0 s_0 + psi_y1 s_1)      d/dx = dpsi_x (psi_y0 s_0 + psi_y1 s_1)
//   d/dy = psi_x (dpsi_y0 s_0 + dpsi_y1 s_1)    d/dz = psi_x  (psi_y0 t_0 + psi_y1 t_1)
// (psi' in grid units, as the reference's pre_dpsi_tensor).  The shares of
// all threads are added in a fixed order in shared memory, four threads per
// (node, output) with compensated (Kahan) sums, in sub-batches of NS nodes (as many as the CTA's threads
// cover).  Window rows (psi and psi' on
// each axis) are evaluated for NB nodes at a time, one thread per (derivative,
// axis, node), a warp sharing the polynomial rows.
// Node row layout (floats):
//   [0, W) psi_z and [W, 2W) dpsi_z in slot rotation (zero outside the stencil)
//   [2W, 2W+16) psi_x, [2W+16, 2W+32) dpsi_x over the region's rows
//   [2W+32, 2W+48) psi_y, [2W+48, 2W+64) dpsi_y over the column pairs (b, b + R/2)
// ---------------------------------------------------------------------------
template <int CUT, int MODE>
struct GradGeom32 {
  typedef LineGeom32<CUT> L;
  static constexpr int NO = (MODE & 1) ? 4 : 3;  // outputs per node: [f,] d/dx, d/dy, d/dz
  static constexpr int NB = 32;                        // nodes per window batch
  static constexpr int NS = L::THREADS / (4 * NO);     // nodes per reduction sub-batch
  static constexpr int WS = 2 * L::W + 64 + 4;         // floats per node row (pad: fewer bank conflicts)
  static constexpr int PR = L::THREADS + 2;            // float2 per share row
  static_assert(NS >= 1 && NO * NS * 4 <= L::THREADS, "four threads per (node, output)");
  static_assert(WS % 4 == 0, "16-byte aligned node rows");
};

template <int CUT, int MODE>
__global__ void __launch_bounds__(LineGeom32<CUT>::THREADS, 3) k_interp_line_g(ConvArgs a) {
  typedef LineGeom32<CUT> G;
  typedef GradGeom32<CUT, MODE> GG;
  constexpr int TL = G::TL, R = G::R, HR = G::HR, W = G::W, NG = G::NG, PS = G::PS, NTH = G::THREADS;
  constexpr int NO = GG::NO, NB = GG::NB, NS = GG::NS, WS = GG::WS, PR = GG::PR;
  constexpr bool ALL_ACTIVE = R * HR == NTH;
  constexpr bool DF = (MODE & 1) != 0;
  __shared__ __align__(16) float s_w[NB][WS];
  __shared__ __align__(16) float2 s_part[NO * NS][PR];
  __shared__ __align__(16) float s_poly[PolyPairs<CUT, 6>::FLOATS];
  __shared__ __align__(16) float4 s_pre[NTH][4];  // prefetched next group of z values, per thread
  __shared__ float s_d[NB][3];
  __shared__ int s_o[NB], s_j[NB], s_slab[NB];
  const Binning &b = a.bin;
  const int sub = blockIdx.x;
  if (sub >= *b.nsub) return;
  const int line = b.sub_tile[sub], first = b.sub_first[sub], cnt = b.sub_cnt[sub];
  if (cnt <= 0) return;  // a line without nodes
  const int t1 = line % b.ntile[1], t0 = line / b.ntile[1];
  const int tid = threadIdx.x;
  const bool active = ALL_ACTIVE || tid < R * HR;
  const int ca = active ? tid / HR : 0, cb = active ? tid % HR : 0;
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  const size_t gx = (size_t)((t0 * TL + ca) % n0) * n1;
  const float2 *grid = (const float2 *)a.grid;
  const float2 *col0 = grid + (gx + (t1 * TL + cb) % n1) * n2;
  const float2 *col1 = grid + (gx + (t1 * TL + cb + HR) % n1) * n2;
  const bool vec = (n2 & 3) == 0;
  const WindowArgs &w = a.w;
  const bool poly = w.poly && w.intpol_order < 0;
  if (poly)  // psi and psi' rows in pairs of stencil points: the polynomial rows of derivatives 0 and 1
    stage_poly_pairs<CUT, NTH, 6>(w.poly, s_poly, tid);
  const float scale = a.use_il ? 0.5f : 1.f;
  float2 *pre = (float2 *)s_pre[tid];

  float2 g0[W], g1[W];  // the two columns' z windows, slot p holds z = p (mod W)
#pragma unroll
  for (int p = 0; p < W; p++) g0[p] = g1[p] = make_float2(0.f, 0.f);
  int zs = -1;
  bool pending = false;

  for (int b0 = 0; b0 < cnt; b0 += NB) {
    const int nb = min(NB, cnt - b0);
    __syncthreads();  // the previous batch's rows are consumed
    if (tid < nb) {
      const float4 r = ((const float4 *)b.rec)[first + b0 + tid];
      s_d[tid][0] = r.x;
      s_d[tid][1] = r.y;
      s_d[tid][2] = r.z;
      const int pk = __float_as_int(r.w);
      s_o[tid] = pk;
      s_slab[tid] = ((pk >> 16) & 0x7fff) >> 2;
      s_j[tid] = b.perm[first + b0 + tid];
    }
    __syncthreads();
    // --- window rows: one thread per (derivative, axis, node) -------------------
    for (int v = tid; v < 2 * 3 * NB; v += NTH) {
      const int e = v / NB, i = v - e * NB, der = e / 3, t = e - 3 * der;
      if (i >= nb) continue;
      float val[CUT];
      window_row_pp_d<CUT>(w, poly, s_poly, der, t, s_d[i][t], val);
      const int pk = s_o[i];
      float *row = s_w[i];
      if (t == 2) {
        const int u2 = (pk >> 16) & 0x7fff;
        float *rz = row + der * W;
#pragma unroll
        for (int c = 0; c < W; c++) rz[(u2 + c) & (W - 1)] = c < CUT ? val[c] : 0.f;
      } else if (t == 0) {
        const int o0 = pk & 0xff;
        float *rx = row + 2 * W + 16 * der;
#pragma unroll
        for (int q = 0; q < 4; q++) ((float4 *)rx)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int c = 0; c < CUT; c++) rx[o0 + c] = val[c];
      } else {
        const int o1 = (pk >> 8) & 0xff;
        float *ry = row + 2 * W + 32 + 16 * der;
#pragma unroll
        for (int q = 0; q < 4; q++) ((float4 *)ry)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int c = 0; c < CUT; c++) {
          const int bc = o1 + c;
          ry[bc < HR ? 2 * bc : 2 * (bc - HR) + 1] = val[c];
        }
      }
    }
    __syncthreads();
    for (int s0 = 0; s0 < nb; s0 += NS) {
      const int ns = min(NS, nb - s0);
      // --- shares of the sub-batch's nodes ---------------------------------------
      for (int i = s0; i < s0 + ns; i++) {
        const int slab = s_slab[i];
        if (slab != zs) {
          if (active) {
            const bool next = pending && slab == zs + 1;
            if (pending) cp_async_wait_all();
#pragma unroll
            for (int q = 0; q < NG; q++) {
              const int zq = 4 * (slab + ((q - slab) & (NG - 1)));
              if (zs < 0 || zq >= 4 * zs + W) {
                if (next) {
                  const float4 *pp = (const float4 *)pre;
                  const float4 u0 = pp[0], u1 = pp[1], u2 = pp[2], u3 = pp[3];
                  g0[4 * q] = make_float2(u0.x, u0.y);
                  g0[4 * q + 1] = make_float2(u0.z, u0.w);
                  g0[4 * q + 2] = make_float2(u1.x, u1.y);
                  g0[4 * q + 3] = make_float2(u1.z, u1.w);
                  g1[4 * q] = make_float2(u2.x, u2.y);
                  g1[4 * q + 1] = make_float2(u2.z, u2.w);
                  g1[4 * q + 2] = make_float2(u3.x, u3.y);
                  g1[4 * q + 3] = make_float2(u3.z, u3.w);
                  if (a.real_only) {
#pragma unroll
                    for (int k = 0; k < 4; k++) g0[4 * q + k].y = g1[4 * q + k].y = 0.f;
                  }
                } else {
                  load_z4(col0, zq, n2, vec, a.real_only, &g0[4 * q]);
                  load_z4(col1, zq, n2, vec, a.real_only, &g1[4 * q]);
                }
              }
            }
            pending = false;
            if (vec) {
              const int zn = wrap_n(4 * slab + W, n2);
              cp_async16(pre, col0 + zn);
              cp_async16(pre + 2, col0 + zn + 2);
              cp_async16(pre + 4, col1 + zn);
              cp_async16(pre + 6, col1 + zn + 2);
              cp_async_commit();
              pending = true;
            }
          }
          zs = slab;
        }
        const float *row = s_w[i];
        const float4 *pz4 = (const float4 *)row, *dz4 = (const float4 *)(row + W);
        float2 sa0 = make_float2(0.f, 0.f), sb0 = sa0, sa1 = sa0, sb1 = sa0;  // psi_z sums, columns 0 / 1
        float2 ta0 = sa0, tb0 = sa0, ta1 = sa0, tb1 = sa0;                    // dpsi_z sums
#pragma unroll
        for (int q = 0; q < NG; q++) {
          const float4 z = pz4[q], d = dz4[q];
          sa0 = __ffma2_rn(g0[4 * q], make_float2(z.x, z.x), sa0);
          sa1 = __ffma2_rn(g1[4 * q], make_float2(z.x, z.x), sa1);
          ta0 = __ffma2_rn(g0[4 * q], make_float2(d.x, d.x), ta0);
          ta1 = __ffma2_rn(g1[4 * q], make_float2(d.x, d.x), ta1);
          sb0 = __ffma2_rn(g0[4 * q + 1], make_float2(z.y, z.y), sb0);
          sb1 = __ffma2_rn(g1[4 * q + 1], make_float2(z.y, z.y), sb1);
          tb0 = __ffma2_rn(g0[4 * q + 1], make_float2(d.y, d.y), tb0);
          tb1 = __ffma2_rn(g1[4 * q + 1], make_float2(d.y, d.y), tb1);
          sa0 = __ffma2_rn(g0[4 * q + 2], make_float2(z.z, z.z), sa0);
          sa1 = __ffma2_rn(g1[4 * q + 2], make_float2(z.z, z.z), sa1);
          ta0 = __ffma2_rn(g0[4 * q + 2], make_float2(d.z, d.z), ta0);
          ta1 = __ffma2_rn(g1[4 * q + 2], make_float2(d.z, d.z), ta1);
          sb0 = __ffma2_rn(g0[4 * q + 3], make_float2(z.w, z.w), sb0);
          sb1 = __ffma2_rn(g1[4 * q + 3], make_float2(z.w, z.w), sb1);
          tb0 = __ffma2_rn(g0[4 * q + 3], make_float2(d.w, d.w), tb0);
          tb1 = __ffma2_rn(g1[4 * q + 3], make_float2(d.w, d.w), tb1);
        }
        const float2 s0v = __fadd2_rn(sa0, sb0), s1v = __fadd2_rn(sa1, sb1);
        const float2 t0v = __fadd2_rn(ta0, tb0), t1v = __fadd2_rn(ta1, tb1);
        const float px = row[2 * W + ca], dpx = row[2 * W + 16 + ca];
        const float2 py = ((const float2 *)(row + 2 * W + 32))[cb], dpy = ((const float2 *)(row + 2 * W + 48))[cb];
        float2 u = __fmul2_rn(s0v, make_float2(py.x, py.x));
        u = __ffma2_rn(s1v, make_float2(py.y, py.y), u);
        float2 v = __fmul2_rn(s0v, make_float2(dpy.x, dpy.x));
        v = __ffma2_rn(s1v, make_float2(dpy.y, dpy.y), v);
        float2 z = __fmul2_rn(t0v, make_float2(py.x, py.x));
        z = __ffma2_rn(t1v, make_float2(py.y, py.y), z);
        const float2 zero = make_float2(0.f, 0.f);
        const int k = i - s0;
        int o = 0;
        if (DF) s_part[(o++) * NS + k][tid] = active ? __fmul2_rn(u, make_float2(px, px)) : zero;
        s_part[(o++) * NS + k][tid] = active ? __fmul2_rn(u, make_float2(dpx, dpx)) : zero;
        s_part[(o++) * NS + k][tid] = active ? __fmul2_rn(v, make_float2(px, px)) : zero;
        s_part[(o++) * NS + k][tid] = active ? __fmul2_rn(z, make_float2(px, px)) : zero;
      }
      __syncthreads();
      // --- sums: four threads per (output, node), a fixed order --------------------
      {
        const int pr = tid >> 2, r = tid & 3;  // pr = output * NS + node
        const int o = pr / NS, k = pr - o * NS;
        float2 sum = make_float2(0.f, 0.f);
        const bool valid = pr < NO * NS && k < ns;
        if (valid) sum = kahan_quarter_sum<NTH>(s_part[pr], r);
        sum.x += __shfl_xor_sync(0xffffffffu, sum.x, 1);
        sum.y += __shfl_xor_sync(0xffffffffu, sum.y, 1);
        sum.x += __shfl_xor_sync(0xffffffffu, sum.x, 2);
        sum.y += __shfl_xor_sync(0xffffffffu, sum.y, 2);
        if (valid && r == 0) {
          const int64_t ind = (int64_t)s_j[s0 + k] * a.stride + a.offset;
          double *out;
          int64_t e;
          if (DF && o == 0) {
            out = a.f_out;
            e = ind;
          } else {
            out = a.grad_out;
            e = 3 * ind + (o - (DF ? 1 : 0));
          }
          const double vr = (double)(sum.x * scale), vi = (double)(sum.y * scale);
          if (a.real_io) {
            if (a.accum) out[e] += vr;
            else out[e] = vr;
          } else {
            double2 *o2 = (double2 *)out + e;
            if (a.accum) {
              double2 t = *o2;
              t.x += vr;
              t.y += vi;
              *o2 = t;
            } else {
              *o2 = make_double2(vr, vi);
            }
          }
        }
      }
      __syncthreads();  // the shares are consumed
    }
  }
  if (pending) cp_async_wait_all();  // no copy outlives the CTA
}

template <int CUT, int MODE>
static void run_interp_line_g(const ConvArgs &a, cudaStream_t s) {
  k_interp_line_g<CUT, MODE><<<a.bin.max_subs, LineGeom32<CUT>::THREADS, 0, s>>>(a);
}

template <int MODE>
static bool interp_line_g_by_cut(const ConvArgs &a, cudaStream_t s) {
  switch (a.w.cut) {
    case 5: run_interp_line_g<5, MODE>(a, s); return true;
    case 7: run_interp_line_g<7, MODE>(a, s); return true;
    case 9: run_interp_line_g<9, MODE>(a, s); return true;
    case 11: run_interp_line_g<11, MODE>(a, s); return true;
    case 13: run_interp_line_g<13, MODE>(a, s); return true;
    default: return false;
  }
}

bool launch_interp_line_g(const ConvArgs &a, int mode, cudaStream_t s) {
  switch (mode) {
    case 2: return interp_line_g_by_cut<2>(a, s);
    case 3: return interp_line_g_by_cut<3>(a, s);
    default: return false;
  }
}

}  // namespace pg
