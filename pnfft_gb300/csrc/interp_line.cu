// interp_line.cu -- interpolation B of the FP32-mixed plans (f only) along
// lines of tiles: the transpose of the spreading of spread_line.cuh, on the
// same binning.
//
// Reference: loop_over_particles_trafo (kernel/ndft-parallel.c:2703-2888)
// with the interpolation loops of kernel/assign.c:667-691.
#include <cuda_runtime.h>

#include "line_f32.cuh"

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
// in shared memory (four threads per node with compensated (Kahan) sums, then
// two shuffles), so a node's result depends only on the node.
// Window values: one thread per (axis, node) evaluates the node's CUT values
// on that axis (a warp shares the axis, so the fitted polynomials'
// coefficients are broadcast reads) into its row: the z row in slot rotation
// (zero outside the stencil), the x row over the region's rows and the y row
// over the region's column pairs.  Nodes of one slab go through the z sums
// in pairs (8 independent FMA chains), and the group of z values that the
// next slab brings in is prefetched with cp.async.
// ---------------------------------------------------------------------------
// z sums of the two columns for one node: 4 independent FFMA2 chains
template <int NG>
__device__ __forceinline__ void zsum(const float2 *g0, const float2 *g1, const float4 *pz4, float2 &s0, float2 &s1) {
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
  s0 = __fadd2_rn(s0a, s0b);
  s1 = __fadd2_rn(s1a, s1b);
}

// the same for two nodes of one slab: 8 independent chains
template <int NG>
__device__ __forceinline__ void zsum2(const float2 *g0, const float2 *g1, const float4 *pa, const float4 *pb,
                                      float2 &a0, float2 &a1, float2 &b0, float2 &b1) {
  float2 a0a = make_float2(0.f, 0.f), a0b = a0a, a1a = a0a, a1b = a0a, b0a = a0a, b0b = a0a, b1a = a0a, b1b = a0a;
#pragma unroll
  for (int q = 0; q < NG; q++) {
    const float4 y = pa[q], z = pb[q];
    a0a = __ffma2_rn(g0[4 * q], make_float2(y.x, y.x), a0a);
    a1a = __ffma2_rn(g1[4 * q], make_float2(y.x, y.x), a1a);
    b0a = __ffma2_rn(g0[4 * q], make_float2(z.x, z.x), b0a);
    b1a = __ffma2_rn(g1[4 * q], make_float2(z.x, z.x), b1a);
    a0b = __ffma2_rn(g0[4 * q + 1], make_float2(y.y, y.y), a0b);
    a1b = __ffma2_rn(g1[4 * q + 1], make_float2(y.y, y.y), a1b);
    b0b = __ffma2_rn(g0[4 * q + 1], make_float2(z.y, z.y), b0b);
    b1b = __ffma2_rn(g1[4 * q + 1], make_float2(z.y, z.y), b1b);
    a0a = __ffma2_rn(g0[4 * q + 2], make_float2(y.z, y.z), a0a);
    a1a = __ffma2_rn(g1[4 * q + 2], make_float2(y.z, y.z), a1a);
    b0a = __ffma2_rn(g0[4 * q + 2], make_float2(z.z, z.z), b0a);
    b1a = __ffma2_rn(g1[4 * q + 2], make_float2(z.z, z.z), b1a);
    a0b = __ffma2_rn(g0[4 * q + 3], make_float2(y.w, y.w), a0b);
    a1b = __ffma2_rn(g1[4 * q + 3], make_float2(y.w, y.w), a1b);
    b0b = __ffma2_rn(g0[4 * q + 3], make_float2(z.w, z.w), b0b);
    b1b = __ffma2_rn(g1[4 * q + 3], make_float2(z.w, z.w), b1b);
  }
  a0 = __fadd2_rn(a0a, a0b);
  a1 = __fadd2_rn(a1a, a1b);
  b0 = __fadd2_rn(b0a, b0b);
  b1 = __fadd2_rn(b1a, b1b);
}

// the thread's share of a node: psi_x[a] (psi_y[b] s0 + psi_y[b + R/2] s1)
template <int W>
__device__ __forceinline__ float2 share(const float *row, int ca, int cb, float2 s0, float2 s1) {
  const float px = row[W + ca];
  const float2 py = ((const float2 *)(row + W + 16))[cb];
  float2 t = __fmul2_rn(s0, make_float2(py.x, py.x));
  t = __ffma2_rn(s1, make_float2(py.y, py.y), t);
  return __fmul2_rn(t, make_float2(px, px));
}

template <int CUT>
__device__ __forceinline__ void interp_line_body(const ConvArgs &a, const int sub) {
  typedef LineGeom32<CUT> G;
  constexpr int TL = G::TL, R = G::R, HR = G::HR, W = G::W, NG = G::NG, NB = G::NB, WS = G::WS, PS = G::PS,
                PR = G::PR, NTH = G::THREADS;
  constexpr bool ALL_ACTIVE = R * HR == NTH;
  __shared__ __align__(16) float s_w[NB][WS];
  __shared__ __align__(16) float2 s_part[NB][PR];
  __shared__ __align__(16) float s_poly[3 * CUT * PS];
  __shared__ __align__(16) float2 s_pre[NTH][8];  // prefetched next group of z values, per thread
  __shared__ float s_d[NB][3];
  __shared__ int s_o[NB], s_j[NB], s_slab[NB];
  const Binning &b = a.bin;
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
  // n2 % 4 == 0: a group of 4 z values is contiguous and 32-byte aligned, and
  // the next slab's group is prefetched with cp.async
  const bool vec = (n2 & 3) == 0;
  const WindowArgs &w = a.w;
  const bool poly = w.poly && w.intpol_order < 0;
  if (poly)
    for (int i = tid; i < 3 * CUT * 4; i += NTH)
      ((float4 *)(s_poly + (i >> 2) * PS))[i & 3] = __ldg((const float4 *)(w.poly + (i >> 2) * kPolyCoef) + (i & 3));
  const float scale = a.use_il ? 0.5f : 1.f;
  float2 *pre = s_pre[tid];

  float2 g0[W], g1[W];  // the two columns' z windows, slot p holds z = p (mod W)
#pragma unroll
  for (int p = 0; p < W; p++) g0[p] = g1[p] = make_float2(0.f, 0.f);
  int zs = -1;          // slab of the window (-1: none loaded)
  bool pending = false;  // a prefetch of the group for slab zs + 1 is in flight

  for (int b0 = 0; b0 < cnt; b0 += NB) {
    const int nb = min(NB, cnt - b0);
    __syncthreads();  // the previous batch's rows and shares are consumed
    // --- stage the node records ------------------------------------------------
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
    // --- window rows: one thread per (axis, node) ----------------------------------
    if (tid < 3 * NB) {
      const int t = tid / NB, i = tid - t * NB;  // a warp shares the axis: broadcast polynomial rows
      if (i < nb) {
        float v[CUT];
        window_row<CUT>(w, poly, s_poly, t, s_d[i][t], v);
        const int pk = s_o[i];
        float *row = s_w[i];
        if (t == 2) {  // z slots in the window's rotation; the W - CUT others are zero
          const int u2 = (pk >> 16) & 0x7fff;
#pragma unroll
          for (int c = 0; c < W; c++) row[(u2 + c) & (W - 1)] = c < CUT ? v[c] : 0.f;
        } else if (t == 0) {  // region rows
          const int o0 = pk & 0xff;
#pragma unroll
          for (int q = 0; q < 4; q++) ((float4 *)(row + W))[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int c = 0; c < CUT; c++) row[W + o0 + c] = v[c];
        } else {  // region columns as (b, b + R/2) pairs
          const int o1 = (pk >> 8) & 0xff;
#pragma unroll
          for (int q = 0; q < 4; q++) ((float4 *)(row + W + 16))[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int c = 0; c < CUT; c++) {
            const int bc = o1 + c;
            row[W + 16 + 2 * (bc < HR ? bc : bc - HR) + (bc < HR ? 0 : 1)] = v[c];
          }
        }
      }
    }
    __syncthreads();
    // --- the z sums of the thread's two columns, nodes of one slab in pairs -------
    for (int i = 0; i < nb;) {
      const int slab = s_slab[i];
      if (slab != zs) {
        if (active) {
          // group q of the new window holds z = 4 (slab + ((q - slab) mod NG))
          const bool next = pending && slab == zs + 1;
          if (pending) cp_async_wait_all();  // also before the slot is refilled after a jump
#pragma unroll
          for (int q = 0; q < NG; q++) {
            const int zq = 4 * (slab + ((q - slab) & (NG - 1)));
            if (zs < 0 || zq >= 4 * zs + W) {
              if (next) {  // the only new group, prefetched
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
          if (vec) {  // the group that the next slab brings in
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
      if (i + 1 < nb && s_slab[i + 1] == slab) {
        float2 a0, a1, c0, c1;
        zsum2<NG>(g0, g1, (const float4 *)s_w[i], (const float4 *)s_w[i + 1], a0, a1, c0, c1);
        const float2 ta = share<W>(s_w[i], ca, cb, a0, a1), tb = share<W>(s_w[i + 1], ca, cb, c0, c1);
        s_part[i][tid] = active ? ta : make_float2(0.f, 0.f);
        s_part[i + 1][tid] = active ? tb : make_float2(0.f, 0.f);
        i += 2;
      } else {
        float2 s0, s1;
        zsum<NG>(g0, g1, (const float4 *)s_w[i], s0, s1);
        const float2 t = share<W>(s_w[i], ca, cb, s0, s1);
        s_part[i][tid] = active ? t : make_float2(0.f, 0.f);
        i += 1;
      }
    }
    __syncthreads();
    // --- the node sums: four threads per node, a fixed order -----------------------
    {
      const int i = tid >> 2, r = tid & 3;
      float2 s = make_float2(0.f, 0.f);
      if (i < nb) s = kahan_quarter_sum<NTH>(s_part[i], r);
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
  if (pending) cp_async_wait_all();  // no copy outlives the CTA
}

template <int CUT>
__global__ void __launch_bounds__(LineGeom32<CUT>::THREADS, 4) k_interp_line(ConvArgs a) {
  interp_line_body<CUT>(a, blockIdx.x);
}

// the sub-problems of several calls of one cutoff in one launch
template <int CUT>
__global__ void __launch_bounds__(LineGeom32<CUT>::THREADS, 4) k_interp_line_multi(MultiConv mc) {
  __shared__ __align__(16) ConvArgs s_args;
  const int item = multi_item(mc, blockIdx.x);
  copy_args(&s_args, mc.args[item]);
  interp_line_body<CUT>(s_args, blockIdx.x - mc.first[item]);
}

template <int CUT>
static void run_interp_line(const ConvArgs &a, cudaStream_t s) {
  k_interp_line<CUT><<<a.bin.max_subs, LineGeom32<CUT>::THREADS, 0, s>>>(a);
}

template <int CUT>
static void run_interp_line_multi(const MultiConv &mc, cudaStream_t s) {
  if (mc.first[mc.n] > 0) k_interp_line_multi<CUT><<<mc.first[mc.n], LineGeom32<CUT>::THREADS, 0, s>>>(mc);
}

bool launch_interp_line_multi(const MultiConv &mc, int cut, cudaStream_t s) {
  switch (cut) {
    case 5: run_interp_line_multi<5>(mc, s); return true;
    case 7: run_interp_line_multi<7>(mc, s); return true;
    case 9: run_interp_line_multi<9>(mc, s); return true;
    case 11: run_interp_line_multi<11>(mc, s); return true;
    case 13: run_interp_line_multi<13>(mc, s); return true;
    default: return false;
  }
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
