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
// z it takes next -- no register moves.  A complete commit at the start of a
// batch once kFlushLineNodes or more nodes ran without a slide bounds the FP32
// summation length in dense clusters (at most NB + kFlushLineNodes - 1 = 127
// nodes per run).
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
__global__ void __launch_bounds__(LineGeom32<CUT>::THREADS, CUT == 11 ? 3 : 4) k_spread_line_f(ConvArgs a) {
  const int sub = blockIdx.x;
#include "spread_line_f_body.inc"
}

// the sub-problems of several calls of one cutoff in one launch
template <int CUT>
__global__ void __launch_bounds__(LineGeom32<CUT>::THREADS, CUT == 11 ? 3 : 4) k_spread_line_f_multi(MultiConv mc) {
  __shared__ __align__(16) ConvArgs s_args;
  const int item = multi_item(mc, blockIdx.x);
  copy_args(&s_args, mc.args[item]);
  const ConvArgs &a = s_args;
  const int sub = blockIdx.x - mc.first[item];
#include "spread_line_f_body.inc"
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
