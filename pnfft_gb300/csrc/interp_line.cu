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
__global__ void __launch_bounds__(LineGeom32<CUT>::THREADS, 4) k_interp_line(ConvArgs a) {
  const int sub = blockIdx.x;
#include "interp_line_body.inc"
}

// the sub-problems of several calls of one cutoff in one launch
template <int CUT>
__global__ void __launch_bounds__(LineGeom32<CUT>::THREADS, 4) k_interp_line_multi(MultiConv mc) {
  __shared__ __align__(16) ConvArgs s_args;
  const int item = multi_item(mc, blockIdx.x);
  copy_args(&s_args, mc.args[item]);
  const ConvArgs &a = s_args;
  const int sub = blockIdx.x - mc.first[item];
#include "interp_line_body.inc"
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
