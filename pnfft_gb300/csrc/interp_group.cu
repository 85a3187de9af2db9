// interp_group.cu -- interpolation B of the FP32-mixed plans (f only) on a
// group-mode binning: one warp per group of nodes with overlapping stencils.
//
// Reference: loop_over_particles_trafo (kernel/ndft-parallel.c:2703-2888)
// with the interpolation loops of kernel/assign.c:667-1159.
#include <cuda_runtime.h>

#include <atomic>

#include "pg_conv.cuh"
#include "pg_kernels.h"
#include "pg_math.cuh"

namespace pg {

// ---------------------------------------------------------------------------
// interpolation B, FP32-mixed, f only, on a group-mode binning.  The nodes
// of one 2x2x4 block of stencil corners come in groups of up to kGroupMax;
// one warp interpolates a whole group, so every grid value read from shared
// memory feeds the sums of all nodes of the group.  The union of the group's
// stencils spans at most (CUT+1) x (CUT+1) x (CUT+3) grid points, CUT <= 13:
// lanes (row = lane/16, col = lane%16) read two z-rows of <= 16 consecutive
// values per step.  Each node's window values are stored shifted to the
// node's offset in the union, in zero-padded rows of 16 (x, y, z), so the
// loops carry no range checks.  Zero-weight terms add exact zeros, so every
// lane holds, for each node, the same partial sum in the same order as the
// lane (l1 parity, z column) of k_interp_tile; a shuffle moves it there and
// the warp reduction is the same, which gives the same bits as
// k_interp_tile<float, CUT, 1>.
// Per CTA: the tile's region, the sub-problem's records and output indices
// and the fitted window polynomials are staged in shared memory, the list
// of groups (a group starts at a record with kGroupBit or at the
// sub-problem's first node) is built with ballots, then each warp takes
// groups round-robin with no global loads: window values into its own
// slots, the stencil sums, and the writes of the group's results.
// ---------------------------------------------------------------------------
template <int CUT>
struct GroupGeom {
  static_assert(CUT + 3 <= 16, "a group's z extent must fit a half-warp");
  static constexpr int R = 8 + CUT - 1, PL = R * R, VOL = R * R * R;
  static constexpr int NV = 3 * CUT;  // psi of one node on the three axes
  static constexpr int NW = 48;       // window slots of one node: x, y, z rows of 16
  static constexpr int PS = 20;       // shared-memory stride of a polynomial row (16 used)
  static constexpr int WARPS = 8, MAXSUB = kGroupSubMax;  // warps per CTA, nodes per sub-problem
  static constexpr size_t SMEM = (size_t)VOL * sizeof(float2) + (size_t)MAXSUB * sizeof(float4) +
                                 (size_t)WARPS * kGroupMax * NW * sizeof(float) + (size_t)NV * PS * sizeof(float) +
                                 (size_t)MAXSUB * sizeof(int) + (MAXSUB + 4) * sizeof(int) + 2 * 32 * sizeof(int);
};

// the stencil sums of a group of G nodes, of which the first g are real
// (window slots wv; the others have zero weights); lane k < g writes the
// result of node k (output index jn of that lane)
template <int CUT, int G>
__device__ __forceinline__ void group_sums(const ConvArgs &a, const float2 *__restrict__ reg, const float *wv,
                                           const int *oy, const int *oz, int x0, int y0, int z0,
                                           int dx, int dy, int dz, int g, int lane, int jn, float scale) {
  typedef GroupGeom<CUT> Gm;
  constexpr int R = Gm::R, PL = Gm::PL, NW = Gm::NW;
  const int row = lane >> 4, col = lane & 15;
  float px[G][16], pz[G];
#pragma unroll
  for (int k = 0; k < G; k++) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float4 t = ((const float4 *)(wv + k * NW))[q];
      px[k][4 * q] = t.x;
      px[k][4 * q + 1] = t.y;
      px[k][4 * q + 2] = t.z;
      px[k][4 * q + 3] = t.w;
    }
    pz[k] = wv[k * NW + 32 + col];
  }
  // complex sums as float2, updated with the paired FMA of sm_100+ (each
  // component rounds like fmaf)
  float2 af[G];
#pragma unroll
  for (int k = 0; k < G; k++) af[k] = make_float2(0.f, 0.f);
  const bool active = col < CUT + dz;
  const float2 *pc = reg + (x0 * R + y0) * R + (z0 + col);
  // the row loop stays rolled (instruction cache)
#pragma unroll 1
  for (int it = 0; it < (CUT + 2) / 2; it++) {
    const int Y = 2 * it + row;  // row of the union
    if (active && Y < CUT + dy) {
      const float2 *p = pc + Y * R;
      // union planes of even and odd L in separate chains: for each node
      // these are its even and odd x planes (in one order or the other, with
      // exact zeros at the ends), as the chains of k_interp_tile; their sum
      // does not depend on the order
      float2 sp[2][G];
#pragma unroll
      for (int k = 0; k < G; k++) sp[0][k] = sp[1][k] = make_float2(0.f, 0.f);
#pragma unroll
      for (int L = 0; L < CUT; L++) {
        const float2 g = p[L * PL];
#pragma unroll
        for (int k = 0; k < G; k++) sp[L & 1][k] = __ffma2_rn(make_float2(px[k][L], px[k][L]), g, sp[L & 1][k]);
      }
      if (dx) {
        const float2 g = p[CUT * PL];
#pragma unroll
        for (int k = 0; k < G; k++)
          sp[CUT & 1][k] = __ffma2_rn(make_float2(px[k][CUT], px[k][CUT]), g, sp[CUT & 1][k]);
      }
#pragma unroll
      for (int k = 0; k < G; k++) {
        const float2 sx = cadd(sp[0][k], sp[1][k]);
        const float wyz = wv[k * NW + 16 + Y] * pz[k];
        af[k] = __ffma2_rn(make_float2(wyz, wyz), sx, af[k]);
      }
    }
  }
  // move each node's partial sums to the lanes of k_interp_tile, then reduce
  // the 2G values together: at each xor distance (16, 8, 4, then 2 and 1)
  // a lane keeps half of its values and adds the partner's copies, so every
  // value sees the pairs of warp_sum, and ends in the lanes whose bits 4..2
  // give its index (2k: re, 2k + 1: im of node k)
  static_assert(G == 4, "the transposed reduction is written for 8 values");
  float v[2 * G];
#pragma unroll
  for (int k = 0; k < G; k++) {
    const int src = (((row + oy[k]) & 1) << 4) + col + oz[k];
    v[2 * k] = __shfl_sync(0xffffffffu, af[k].x, src & 31);
    v[2 * k + 1] = __shfl_sync(0xffffffffu, af[k].y, src & 31);
    if (col >= CUT) v[2 * k] = v[2 * k + 1] = 0.f;
  }
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  float u[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const float send = b4 ? v[j] : v[4 + j];
    const float keep = b4 ? v[4 + j] : v[j];
    u[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
  float w2[2];
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const float send = b3 ? u[j] : u[2 + j];
    const float keep = b3 ? u[2 + j] : u[j];
    w2[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  float x = (b2 ? w2[1] : w2[0]) + __shfl_xor_sync(0xffffffffu, b2 ? w2[0] : w2[1], 4);
  x += __shfl_xor_sync(0xffffffffu, x, 2);
  x += __shfl_xor_sync(0xffffffffu, x, 1);
  // lane k < g writes node k: re from lane 8k, im from lane 8k + 4
  const float r = __shfl_sync(0xffffffffu, x, (8 * lane) & 31);
  const float im = __shfl_sync(0xffffffffu, x, (8 * lane + 4) & 31);
  if (lane < g) {
    const int64_t e = (int64_t)jn * a.stride + a.offset;
    const double vr = (double)(r * scale), vi = (double)(im * scale);
    if (a.real_io) {
      if (a.accum) a.f_out[e] += vr;
      else a.f_out[e] = vr;
    } else {
      double2 *o2 = (double2 *)a.f_out + e;
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

template <int CUT>
__global__ void __launch_bounds__(256, 2) k_interp_group(ConvArgs a) {
  typedef GroupGeom<CUT> Gm;
  constexpr int R = Gm::R, VOL = Gm::VOL, NV = Gm::NV, NW = Gm::NW, PS = Gm::PS, MAXSUB = Gm::MAXSUB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *reg = (float2 *)smem_raw;
  float4 *s_rec = (float4 *)(reg + VOL);                   // [MAXSUB] node records
  float *s_wv = (float *)(s_rec + MAXSUB);                 // [WARPS][kGroupMax][NW] window slots
  float *s_poly = s_wv + Gm::WARPS * kGroupMax * NW;       // [NV][PS] polynomial rows
  int *s_perm = (int *)(s_poly + NV * PS);                 // [MAXSUB] output indices
  int *s_item = s_perm + MAXSUB;                           // [MAXSUB + 1] group starts
  unsigned *s_mask = (unsigned *)(s_item + MAXSUB + 4);    // [32]
  int *s_off = (int *)(s_mask + 32);                       // [32]
  const Binning &b = a.bin;
  const int sub = blockIdx.x;
  if (sub >= *b.nsub) return;
  const int tile = b.sub_tile[sub], first = b.sub_first[sub], cnt = min(b.sub_cnt[sub], MAXSUB);
  if (cnt <= 0) return;
  int base[3];
  tile_base(b, tile, base);
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  const WindowArgs &w = a.w;
  const bool poly = w.poly && w.intpol_order < 0;
  const float2 *grid = (const float2 *)a.grid;
  load_region<R>(reg, grid, base, n0, n1, n2, a.real_only);
  if (poly)
    for (int i = tid; i < NV * 4; i += blockDim.x)
      ((float4 *)(s_poly + (i >> 2) * PS))[i & 3] = __ldg((const float4 *)(w.poly + (i >> 2) * kPolyCoef) + (i & 3));
  // records, output indices and the group starts (flagged records and the
  // first node), one warp per chunk of 32 nodes
  const float4 *rec = (const float4 *)b.rec;
  const int nch = (cnt + 31) >> 5;
  for (int c = warp; c < nch; c += nwarp) {
    const int i = (c << 5) + lane;
    bool st = false;
    if (i < cnt) {
      const float4 r = rec[first + i];
      s_rec[i] = r;
      s_perm[i] = b.perm[first + i];
      st = i == 0 || (__float_as_int(r.w) & kGroupBit);
    }
    const unsigned m = __ballot_sync(0xffffffffu, st);
    if (lane == 0) s_mask[c] = m;
  }
  __syncthreads();
  if (warp == 0) {
    const int v = lane < nch ? __popc(s_mask[lane]) : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    s_off[lane] = x - v;
    if (lane == 31) s_item[MAXSUB + 1] = x;
  }
  __syncthreads();
  for (int c = warp; c < nch; c += nwarp) {
    const unsigned m = s_mask[c];
    if ((m >> lane) & 1u) s_item[s_off[c] + __popc(m & ((1u << lane) - 1u))] = (c << 5) + lane;
  }
  const int nitem = s_item[MAXSUB + 1];
  __syncthreads();
  if (tid == 0) s_item[nitem] = cnt;
  __syncthreads();

  float *wv = s_wv + warp * kGroupMax * NW;
  const float scale = a.use_il ? 0.5f : 1.f;
  for (int it = warp; it < nitem; it += nwarp) {
    // 1..kGroupMax by construction of the group-start flags (clamped so that a
    // malformed list can never index past the warp's slots)
    const int i0 = s_item[it], g = min(s_item[it + 1] - i0, kGroupMax);
    const float4 *nd = s_rec + i0;
    const int jn = lane < g ? s_perm[i0 + lane] : 0;
    // corners: the union's lowest corner and each node's offset in it (y, z;
    // the x offset is in the window rows)
    int oy[kGroupMax], oz[kGroupMax];
    int x0 = 255, y0 = 255, z0 = 255, x1 = 0, y1 = 0, z1 = 0;
#pragma unroll
    for (int k = 0; k < kGroupMax; k++) {
      int o[3];
      unpack_corner(__float_as_int(nd[k < g ? k : 0].w), o);
      oy[k] = o[1];
      oz[k] = o[2];
      x0 = min(x0, o[0]);
      x1 = max(x1, o[0]);
      y0 = min(y0, o[1]);
      y1 = max(y1, o[1]);
      z0 = min(z0, o[2]);
      z1 = max(z1, o[2]);
    }
#pragma unroll
    for (int k = 0; k < kGroupMax; k++) {
      oy[k] -= y0;
      oz[k] -= z0;
    }
    // window values, shifted into zeroed slots (also the slots of the
    // zero-weight nodes that pad a group to kGroupMax)
    for (int v = lane; v < kGroupMax * (NW / 4); v += 32) ((float4 *)wv)[v] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    // (node k, value e) pairs over the lanes; value e is stencil point e % CUT
    // on axis e / CUT, stored at its offset in the union
    for (int v = lane; v < g * NV; v += 32) {
      const int k = v / NV, e = v - k * NV, t = e / CUT, sidx = e - t * CUT;
      const float4 r = nd[k];
      const float dist = t == 0 ? r.x : (t == 1 ? r.y : r.z);
      const int sh = ((__float_as_int(r.w) >> (8 * t)) & 0xff) - (t == 0 ? x0 : (t == 1 ? y0 : z0));
      float val;
      if (poly && !(w.kind == WIN_BESSEL_I0 && sidx == 0 && dist == 0.f)) {
        const float4 *rw = (const float4 *)(s_poly + e * PS);
        val = w.poly_ncoef <= 12 ? poly_horner12(rw[0], rw[1], rw[2], dist - 0.5f)
                                 : poly_horner(rw[0], rw[1], rw[2], rw[3], dist - 0.5f);
      } else {
        float out[3];
        window_point<float>(w, t, sidx, dist, 0, out);
        val = out[0];
      }
      wv[k * NW + t * 16 + sidx + sh] = val;
    }
    __syncwarp();
    const int dx = x1 - x0, dy = y1 - y0, dz = z1 - z0;  // <= 1, 1, 3
    // one size of the sums keeps the hot code in the instruction cache;
    // smaller groups are padded with zero-weight nodes
    group_sums<CUT, kGroupMax>(a, reg, wv, oy, oz, x0, y0, z0, dx, dy, dz, g, lane, jn, scale);
    __syncwarp();  // the group's slots are free
  }
}

template <int CUT>
static void run_interp_group(const ConvArgs &a, cudaStream_t s) {
  const size_t sm = GroupGeom<CUT>::SMEM;
  static std::atomic<unsigned long long> attr_done{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(attr_done.load() & bit)) {
    cudaFuncSetAttribute(k_interp_group<CUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr_done.fetch_or(bit);
  }
  k_interp_group<CUT><<<a.bin.max_subs, GroupGeom<CUT>::WARPS * 32, sm, s>>>(a);
}

bool launch_interp_group(const ConvArgs &a, cudaStream_t s) {
  switch (a.w.cut) {
    case 5: run_interp_group<5>(a, s); return true;
    case 7: run_interp_group<7>(a, s); return true;
    case 9: run_interp_group<9>(a, s); return true;
    case 11: run_interp_group<11>(a, s); return true;
    case 13: run_interp_group<13>(a, s); return true;
    default: return false;
  }
}

}  // namespace pg
