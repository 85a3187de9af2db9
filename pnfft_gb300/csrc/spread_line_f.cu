// spread_line_f.cu -- spreading B^T of the FP32-mixed plans (f only, no
// gradient input) along lines of tiles, on the line binning.
//
// Reference: loop_over_particles_adj (kernel/ndft-parallel.c:2890-3009) with
// the spreading loop of kernel/assign.c:478-499.
#include <cuda_runtime.h>

#include "line_f32.cuh"

namespace pg {

// ---------------------------------------------------------------------------
// Geometry and the rotating z window as in line_f32.cuh.  Each thread keeps
// its two columns' W accumulators in registers, in slot rotation.  A node's
// update is
//   acc_c[p] += (f psi_x[a]) psi_y[b_c] * psi_z'[p]     (p = 0 .. W-1)
// with psi_z' the node's z row in slot rotation (zero outside the stencil):
// one FFMA2 per slot and column, no coverage tests (uncovered columns add
// exact zeros).  When a node lies in a later slab, every group of 4 slots
// whose z leaves the window is final for this CTA: it is committed to the
// grid with vector atomics (all-zero pairs are skipped) and cleared for the
// z it takes next -- no register moves.  A complete commit after kFlushLineNodes
// nodes without a slide bounds the FP32 summation length in dense clusters.
// Per batch of NB nodes one thread per (axis, node) evaluates the node's
// CUT window values on that axis and writes the node's rows: the z row, the
// x row times f (complex) over the region's rows, and the y row over the
// region's column pairs, zeros elsewhere.
// ---------------------------------------------------------------------------
constexpr int kFlushLineNodes = 64;

template <int CUT>
struct SpreadGeom32 {
  typedef LineGeom32<CUT> L;
  static constexpr int NB = 64;                  // nodes per batch
  static constexpr int WS = L::W + 48 + 4;       // z slots, f psi_x (16 complex), psi_y pairs (16), pad
  static_assert(WS % 4 == 0, "16-byte aligned node rows");
};

// adds v[0..3] (4 consecutive z from z0, wrapped) into a grid column
__device__ __forceinline__ void commit_z4(float2 *col, int z0, int n2, bool vec, const float2 *v) {
  if (vec) {  // contiguous and 32-byte aligned
    float2 *p = col + wrap_n(z0, n2);
    if (v[0].x != 0.f || v[0].y != 0.f || v[1].x != 0.f || v[1].y != 0.f)
      atomicAdd((float4 *)p, make_float4(v[0].x, v[0].y, v[1].x, v[1].y));
    if (v[2].x != 0.f || v[2].y != 0.f || v[3].x != 0.f || v[3].y != 0.f)
      atomicAdd((float4 *)(p + 2), make_float4(v[2].x, v[2].y, v[3].x, v[3].y));
  } else {
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (v[k].x != 0.f || v[k].y != 0.f) atomicAdd(col + wrap_n(z0 + k, n2), v[k]);
  }
}

template <int CUT>
__device__ __forceinline__ void spread_line_f_body(const ConvArgs &a, const int sub) {
  typedef LineGeom32<CUT> G;
  constexpr int TL = G::TL, R = G::R, HR = G::HR, W = G::W, NG = G::NG, PS = G::PS, NTH = G::THREADS;
  constexpr int NB = SpreadGeom32<CUT>::NB, WS = SpreadGeom32<CUT>::WS;
  constexpr bool ALL_ACTIVE = R * HR == NTH;
  __shared__ __align__(16) float s_w[NB][WS];
  __shared__ __align__(16) float s_poly[3 * CUT * PS];
  __shared__ float s_d[NB][3];
  __shared__ float2 s_f[NB];
  __shared__ int s_o[NB], s_slab[NB];
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
  float2 *grid = (float2 *)a.grid;
  float2 *col0 = grid + (gx + (t1 * TL + cb) % n1) * n2;
  float2 *col1 = grid + (gx + (t1 * TL + cb + HR) % n1) * n2;
  const bool vec = (n2 & 3) == 0;
  const WindowArgs &w = a.w;
  const bool poly = w.poly && w.intpol_order < 0;
  if (poly)
    for (int i = tid; i < 3 * CUT * 4; i += NTH)
      ((float4 *)(s_poly + (i >> 2) * PS))[i & 3] = __ldg((const float4 *)(w.poly + (i >> 2) * kPolyCoef) + (i & 3));
  const float scale = a.use_il ? 0.5f : 1.f;

  float2 acc0[W], acc1[W];  // the two columns' z windows, slot p holds z = p (mod W)
#pragma unroll
  for (int p = 0; p < W; p++) acc0[p] = acc1[p] = make_float2(0.f, 0.f);
  int zs = -1, since = 0;
  // commits (and clears) the groups of the window of slab zs whose z is below zmin
  auto commit = [&](int zmin) {
#pragma unroll
    for (int q = 0; q < NG; q++) {
      const int zq = 4 * (zs + ((q - zs) & (NG - 1)));
      if (zq < zmin) {
        if (active) {
          commit_z4(col0, zq, n2, vec, &acc0[4 * q]);
          commit_z4(col1, zq, n2, vec, &acc1[4 * q]);
        }
#pragma unroll
        for (int k = 0; k < 4; k++) acc0[4 * q + k] = acc1[4 * q + k] = make_float2(0.f, 0.f);
      }
    }
  };

  for (int b0 = 0; b0 < cnt; b0 += NB) {
    const int nb = min(NB, cnt - b0);
    __syncthreads();  // the previous batch's rows are consumed
    // --- stage the node records and values -------------------------------------
    for (int i = tid; i < nb; i += NTH) {
      const int q = first + b0 + i;
      const float4 r = ((const float4 *)b.rec)[q];
      s_d[i][0] = r.x;
      s_d[i][1] = r.y;
      s_d[i][2] = r.z;
      const int pk = __float_as_int(r.w);
      s_o[i] = pk;
      s_slab[i] = ((pk >> 16) & 0x7fff) >> 2;
      const int64_t ind = (int64_t)b.perm[q] * a.stride + a.offset;
      float2 v;
      if (a.real_io) {
        v = make_float2((float)a.f_in[ind], 0.f);
      } else {
        const double2 f = ((const double2 *)a.f_in)[ind];
        v = make_float2((float)f.x, (float)f.y);
      }
      s_f[i] = make_float2(v.x * scale, v.y * scale);
    }
    __syncthreads();
    // --- node rows: one thread per (axis, node) -----------------------------------
    for (int v = tid; v < 3 * NB; v += NTH) {
      const int t = v / NB, i = v - t * NB;  // a warp shares the axis: broadcast polynomial rows
      if (i >= nb) continue;
      float val[CUT];
      window_row<CUT>(w, poly, s_poly, t, s_d[i][t], val);
      const int pk = s_o[i];
      float *row = s_w[i];
      if (t == 2) {  // z slots in the window's rotation; the W - CUT others are zero
        const int u2 = (pk >> 16) & 0x7fff;
#pragma unroll
        for (int c = 0; c < W; c++) row[(u2 + c) & (W - 1)] = c < CUT ? val[c] : 0.f;
      } else if (t == 0) {  // f psi_x over the region's rows (complex)
        const int o0 = pk & 0xff;
        const float2 f = s_f[i];
        float2 *rx = (float2 *)(row + W);
#pragma unroll
        for (int q = 0; q < 8; q++) ((float4 *)rx)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int c = 0; c < CUT; c++) rx[o0 + c] = make_float2(f.x * val[c], f.y * val[c]);
      } else {  // psi_y over the region's columns as (b, b + R/2) pairs
        const int o1 = (pk >> 8) & 0xff;
        float *ry = row + W + 32;
#pragma unroll
        for (int q = 0; q < 4; q++) ((float4 *)ry)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int c = 0; c < CUT; c++) {
          const int bc = o1 + c;
          ry[2 * (bc < HR ? bc : bc - HR) + (bc < HR ? 0 : 1)] = val[c];
        }
      }
    }
    __syncthreads();
    // --- accumulate, sliding the window ------------------------------------------------
    if (since >= kFlushLineNodes && zs >= 0) {
      commit(4 * zs + W);  // everything: bounds the summation length
      since = 0;
    }
    for (int i = 0; i < nb; i++) {
      const int slab = s_slab[i];
      if (slab != zs) {
        if (zs >= 0) commit(4 * slab);  // the groups that leave the window
        zs = slab;
        since = 0;
      }
      since++;
      const float *row = s_w[i];
      const float2 fa = ((const float2 *)(row + W))[ca];
      const float2 py = ((const float2 *)(row + W + 32))[cb];
      const float2 h0 = __fmul2_rn(fa, make_float2(py.x, py.x)), h1 = __fmul2_rn(fa, make_float2(py.y, py.y));
      const float4 *pz4 = (const float4 *)row;
#pragma unroll
      for (int q = 0; q < NG; q++) {
        const float4 z = pz4[q];
        acc0[4 * q] = __ffma2_rn(h0, make_float2(z.x, z.x), acc0[4 * q]);
        acc1[4 * q] = __ffma2_rn(h1, make_float2(z.x, z.x), acc1[4 * q]);
        acc0[4 * q + 1] = __ffma2_rn(h0, make_float2(z.y, z.y), acc0[4 * q + 1]);
        acc1[4 * q + 1] = __ffma2_rn(h1, make_float2(z.y, z.y), acc1[4 * q + 1]);
        acc0[4 * q + 2] = __ffma2_rn(h0, make_float2(z.z, z.z), acc0[4 * q + 2]);
        acc1[4 * q + 2] = __ffma2_rn(h1, make_float2(z.z, z.z), acc1[4 * q + 2]);
        acc0[4 * q + 3] = __ffma2_rn(h0, make_float2(z.w, z.w), acc0[4 * q + 3]);
        acc1[4 * q + 3] = __ffma2_rn(h1, make_float2(z.w, z.w), acc1[4 * q + 3]);
      }
    }
  }
  // --- commit the last window ---------------------------------------------------------
  if (zs >= 0) commit(4 * zs + W);
}

template <int CUT>
__global__ void __launch_bounds__(LineGeom32<CUT>::THREADS, CUT == 11 ? 3 : 4) k_spread_line_f(ConvArgs a) {
  spread_line_f_body<CUT>(a, blockIdx.x);
}

// the sub-problems of several calls of one cutoff in one launch
template <int CUT>
__global__ void __launch_bounds__(LineGeom32<CUT>::THREADS, CUT == 11 ? 3 : 4) k_spread_line_f_multi(MultiConv mc) {
  __shared__ __align__(16) ConvArgs s_args;
  const int item = multi_item(mc, blockIdx.x);
  copy_args(&s_args, mc.args[item]);
  spread_line_f_body<CUT>(s_args, blockIdx.x - mc.first[item]);
}

template <int CUT>
static void run_spread_line_f(const ConvArgs &a, cudaStream_t s) {
  k_spread_line_f<CUT><<<a.bin.max_subs, LineGeom32<CUT>::THREADS, 0, s>>>(a);
}

template <int CUT>
static void run_spread_line_f_multi(const MultiConv &mc, cudaStream_t s) {
  if (mc.first[mc.n] > 0) k_spread_line_f_multi<CUT><<<mc.first[mc.n], LineGeom32<CUT>::THREADS, 0, s>>>(mc);
}

bool launch_spread_line_f_multi(const MultiConv &mc, int cut, cudaStream_t s) {
  switch (cut) {
    case 5: run_spread_line_f_multi<5>(mc, s); return true;
    case 7: run_spread_line_f_multi<7>(mc, s); return true;
    case 9: run_spread_line_f_multi<9>(mc, s); return true;
    case 11: run_spread_line_f_multi<11>(mc, s); return true;
    case 13: run_spread_line_f_multi<13>(mc, s); return true;
    default: return false;
  }
}

bool launch_spread_line_f(const ConvArgs &a, cudaStream_t s) {
  switch (a.w.cut) {
    case 5: run_spread_line_f<5>(a, s); return true;
    case 7: run_spread_line_f<7>(a, s); return true;
    case 9: run_spread_line_f<9>(a, s); return true;
    case 11: run_spread_line_f<11>(a, s); return true;
    case 13: run_spread_line_f<13>(a, s); return true;
    default: return false;
  }
}

}  // namespace pg
