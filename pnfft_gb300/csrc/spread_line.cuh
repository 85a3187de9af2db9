// spread_line.cuh -- spreading B^T along lines of tiles; instantiated per
// precision in spread_line_f32.cu and spread_line_f64.cu.
//
// Reference: loop_over_particles_adj (kernel/ndft-parallel.c:2890-3009) with
// the spreading loops of kernel/assign.c:478-664.
#pragma once
#include <cuda_runtime.h>

#include "pg_conv.cuh"
#include "pg_kernels.h"
#include "pg_math.cuh"

namespace pg {

// vector loads of a staged row
template <typename T, int N>
__device__ __forceinline__ void load_row(const T *p, T *v);
template <int N>
__device__ __forceinline__ void load_row(const float *p, float *v) {
#pragma unroll
  for (int q = 0; q < N / 4; q++) {
    float4 t = ((const float4 *)p)[q];
    v[4 * q] = t.x;
    v[4 * q + 1] = t.y;
    v[4 * q + 2] = t.z;
    v[4 * q + 3] = t.w;
  }
}
template <int N>
__device__ __forceinline__ void load_row(const double *p, double *v) {
#pragma unroll
  for (int q = 0; q < N / 2; q++) {
    double2 t = ((const double2 *)p)[q];
    v[2 * q] = t.x;
    v[2 * q + 1] = t.y;
  }
}

// ---------------------------------------------------------------------------
// spreading B^T along lines of tiles.  One CTA takes the nodes of one line
// of 4x4x4-cell tiles running along axis 2 (the sort keeps them consecutive
// and in slab order, slab = u2/4), or a run of at most sub_max of them.
// The (3+cut)^2 region of the line in axes 0, 1 is split into column pairs:
// thread (a, b) owns the columns (a, b) and (a, b + R/2), and keeps W = 3+cut
// consecutive z values of each in registers, aligned to the slab of the
// current node.  The node's z window row (cut values at offset u2 mod 4, zero
// elsewhere) is staged per node, so each update is a branch-free W-long FMA
// run, and the node decode and the psi_x / psi_z loads serve both columns:
//   acc[z] += f psi_x[a-o0] psi_y[b-o1] * psi_z[z-o2]
// With f only (no gradient input) the node's rows are staged as f psi_x and
// psi_y over the whole region (zero outside the node's stencil), so the
// update of a thread has no coverage test at all; uncovered columns add
// exact zeros.
// When a node lies in a later slab the window slides: its first 4 values
// are final for this CTA and are committed with vector atomics (zeros are
// skipped).  Each z value of a column is therefore committed once per line
// rather than once per tile.  A complete flush after kFlushNodes nodes since
// the last slide bounds the FP32 summation length in dense clusters.
// ---------------------------------------------------------------------------
template <int CUT>
struct LineGeom {
  static constexpr int TL = 4;                   // tile edge in every axis
  static constexpr int R = TL + CUT - 1;         // region edge in axes 0, 1 (even)
  static constexpr int HR = R / 2;               // column pairs per region row
  static constexpr int W = TL + CUT - 1;         // z window (even)
  static constexpr int WP = (W + 3) / 4 * 4;     // padded z row
  static constexpr int CP = (CUT + 3) / 4 * 4;   // padded x / y rows
  static constexpr int WREC = WP + 2 * CP;
  static constexpr int THREADS = (R * HR + 31) / 32 * 32;
};
constexpr int kFlushNodes = 256;

// z mod n2 for 0 <= z (z < 2 n2 in all but the smallest grids: one subtraction)
__device__ __forceinline__ int wrap_z(int z, int n2) {
  if (z >= n2) z -= n2;
  if (z >= n2) z %= n2;
  return z;
}
// adds (r0 + i i0) at z and (r1 + i i1) at z+1 of one grid column (z even)
__device__ __forceinline__ void commit_pair(float2 *col, int z, int n2, bool vec, float r0, float i0, float r1,
                                            float i1) {
  if (r0 == 0.f && i0 == 0.f && r1 == 0.f && i1 == 0.f) return;
  if (vec) {
    atomicAdd((float4 *)(col + wrap_z(z, n2)), make_float4(r0, i0, r1, i1));
  } else {
    if (r0 != 0.f || i0 != 0.f) atomicAdd(col + wrap_z(z, n2), make_float2(r0, i0));
    if (r1 != 0.f || i1 != 0.f) atomicAdd(col + wrap_z(z + 1, n2), make_float2(r1, i1));
  }
}
__device__ __forceinline__ void commit_pair(double2 *col, int z, int n2, bool, double r0, double i0, double r1,
                                            double i1) {
  if (r0 != 0.0 || i0 != 0.0) atomic_add_grid(col + wrap_z(z, n2), make_double2(r0, i0));
  if (r1 != 0.0 || i1 != 0.0) atomic_add_grid(col + wrap_z(z + 1, n2), make_double2(r1, i1));
}

// acc += (hr + i hi) * p: the paired FMA of sm_100+ in FP32 (each component
// rounds like fmaf), two FMAs in FP64
__device__ __forceinline__ void acc_fma(float2 &acc, float hr, float hi, float p) {
  acc = __ffma2_rn(make_float2(hr, hi), make_float2(p, p), acc);
}
__device__ __forceinline__ void acc_fma(double2 &acc, double hr, double hi, double p) {
  acc.x = fma(hr, p, acc.x);
  acc.y = fma(hi, p, acc.y);
}

template <typename T, int CUT, int MODE>
__global__ void __launch_bounds__(LineGeom<CUT>::THREADS, sizeof(T) == 4 ? ((MODE & 2) ? 4 : 5) : 1)
    k_spread_line(ConvArgs a) {
  typedef typename Cplx<T>::type C;
  typedef LineGeom<CUT> G;
  constexpr int TL = G::TL, R = G::R, HR = G::HR, W = G::W, WP = G::WP, CP = G::CP, WREC = G::WREC;
  constexpr bool DF = (MODE & 1) != 0, DG = (MODE & 2) != 0;
  constexpr int NDER = DG ? 1 : 0;
  constexpr int NB = sizeof(T) == 4 ? 64 : 32;  // nodes per batch
  // f only: [pz (WP)][f psi_x at region row a (R complex)][psi_y at region column b (R)],
  // each part a multiple of 4 values so that every row stays 16-byte aligned
  constexpr bool FONLY = !DG;
  constexpr int R4 = (R + 3) / 4 * 4;
  constexpr int WF = WP + 3 * R4;
  static_assert(WP % 4 == 0 && WF % 4 == 0, "16-byte aligned node rows");
  constexpr int WSZ0 = FONLY ? WF : 2 * WREC;
  constexpr int WSZ = (WSZ0 * sizeof(T) / 16) % 2 ? WSZ0 : WSZ0 + 16 / (int)sizeof(T);
  // per node: [pz (WP)][px (CP)][py (CP)] and, with DG, the same for the derivatives
  __shared__ __align__(16) T s_w[NB][WSZ];
  __shared__ T s_v[NB][8];  // f re/im, g0..g2 re/im (scaled)
  __shared__ T s_d[NB][3];
  __shared__ int s_o[NB];
  const Binning &b = a.bin;
  const int sub = blockIdx.x;
  if (sub >= *b.nsub) return;
  const int line = b.sub_tile[sub], first = b.sub_first[sub], cnt = b.sub_cnt[sub];
  if (cnt <= 0) return;  // a line without nodes
  const int t1 = line % b.ntile[1], t0 = line / b.ntile[1];
  const int tid = threadIdx.x, nth = blockDim.x;
  const bool active = tid < R * HR;
  const int ca = active ? tid / HR : 0, cb = active ? tid % HR : 0;
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  const size_t gx = (size_t)((t0 * TL + ca) % n0) * n1;
  C *col[2] = {(C *)a.grid + (gx + (t1 * TL + cb) % n1) * n2, (C *)a.grid + (gx + (t1 * TL + cb + HR) % n1) * n2};
  const bool vec = (n2 & 1) == 0;
  C acc[2][W];  // the two columns' z windows (re, im)
  const C zero = {(T)0, (T)0};
#pragma unroll
  for (int c = 0; c < 2; c++)
#pragma unroll
    for (int z = 0; z < W; z++) acc[c][z] = zero;
  int zslab = -1, since = 0;
  const T scale = a.use_il ? (T)0.5 : (T)1;
  // commit values [z0, z1) of both columns at grid z = zb + z
  auto commit = [&](int zb, int z0, int z1) {
#pragma unroll
    for (int c = 0; c < 2; c++)
#pragma unroll
      for (int z = 0; z < W; z += 2)
        if (z >= z0 && z < z1)
          commit_pair(col[c], zb + z, n2, vec, acc[c][z].x, acc[c][z].y, acc[c][z + 1].x, acc[c][z + 1].y);
  };
  for (int b0 = 0; b0 < cnt; b0 += NB) {
    const int nb = min(NB, cnt - b0);
    __syncthreads();
    // --- stage node data and clear the z rows ---------------------------------
    for (int i = tid; i < nb; i += nth) {
      const int q = first + b0 + i;
      T d[3];
      int pk;
      load_rec_raw(b.rec, q, d, &pk);
      s_d[i][0] = d[0];
      s_d[i][1] = d[1];
      s_d[i][2] = d[2];
      s_o[i] = pk;
      const int64_t ind = (int64_t)b.perm[q] * a.stride + a.offset;
      T v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (DF) {
        if (a.real_io) v[0] = (T)a.f_in[ind];
        else {
          double2 f = ((const double2 *)a.f_in)[ind];
          v[0] = (T)f.x;
          v[1] = (T)f.y;
        }
      }
      if (DG) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
          if (a.real_io) v[2 + 2 * c] = (T)a.grad_in[3 * ind + c];
          else {
            double2 g = ((const double2 *)a.grad_in)[3 * ind + c];
            v[2 + 2 * c] = (T)g.x;
            v[3 + 2 * c] = (T)g.y;
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 8; c++) s_v[i][c] = v[c] * scale;
    }
    if (FONLY) {
      for (int v = tid; v < nb * WF; v += nth) {
        const int i = v / WF, z = v - i * WF;
        s_w[i][z] = (T)0;
      }
    } else {
      for (int v = tid; v < nb * WP; v += nth) {
        const int i = v / WP, z = v - i * WP;
        s_w[i][z] = (T)0;
        s_w[i][WREC + z] = (T)0;
      }
    }
    __syncthreads();
    // --- window values: all threads over (node, axis, stencil point) ------------
    // node-fastest (broadcast polynomial rows); the odd row stride in 16-byte
    // units keeps these stores to at most 4-way bank conflicts
    // one stencil point's window values into the node's row
    auto put = [&](int i, int t, int sidx, const T *out) {
      if (FONLY) {
        const int pk = s_o[i];
        if (t == 2) {
          s_w[i][((pk >> 16) & (TL - 1)) + sidx] = out[0];
        } else if (t == 1) {
          s_w[i][WP + 2 * R4 + ((pk >> 8) & 0xff) + sidx] = out[0];
        } else {
          // f psi_x, the product fr = psi_x f of the covered-column form
          const int r = (pk & 0xff) + sidx;
          s_w[i][WP + 2 * r] = out[0] * s_v[i][0];
          s_w[i][WP + 2 * r + 1] = out[0] * s_v[i][1];
        }
      } else {
        const int pos = (t == 2) ? ((s_o[i] >> 16) & (TL - 1)) + sidx : WP + t * CP + sidx;
        s_w[i][pos] = out[0];
        s_w[i][WREC + pos] = out[1];
      }
    };
    bool paired = false;
    if constexpr (sizeof(T) == 4) {
      // fitted FP32 polynomials: two stencil points per paired FMA
      if (a.w.poly_pp && a.w.intpol_order < 0) {
        paired = true;
        constexpr int NP = (CUT + 1) / 2;
        for (int v = tid; v < NB * 3 * NP; v += nth) {
          const int e2 = v / NB, i = v - e2 * NB;
          if (i >= nb) continue;
          const int t = e2 / NP, cp = e2 - t * NP;
          const float dist = s_d[i][t];
          float2 h[2];
          window_pair(a.w, t, cp, dist, NDER, h);
          T o0[2] = {h[0].x, NDER ? h[1].x : 0.f}, o1[2] = {h[0].y, NDER ? h[1].y : 0.f};
          if (a.w.kind == WIN_BESSEL_I0 && cp == 0 && dist == 0.f) {  // evaluated by the formula there
            T out[3];
            window_point<T>(a.w, t, 0, dist, NDER, out);
            o0[0] = out[0];
            if (NDER) o0[1] = out[1];
          }
          put(i, t, 2 * cp, o0);
          if (2 * cp + 1 < CUT) put(i, t, 2 * cp + 1, o1);
        }
      }
    }
    if (!paired) {
#pragma unroll 4  // independent polynomial chains per thread
      for (int v = tid; v < NB * 3 * CUT; v += nth) {
        const int e = v / NB, i = v - e * NB;
        if (i >= nb) continue;
        const int t = e / CUT, sidx = e - t * CUT;
        T out[3];
        window_point<T>(a.w, t, sidx, s_d[i][t], NDER, out);
        put(i, t, sidx, out);
      }
    }
    __syncthreads();
    // --- accumulate, sliding the z window ----------------------------------------
    if (since >= kFlushNodes) {
      commit(zslab * TL, 0, W);
#pragma unroll
      for (int c = 0; c < 2; c++)
#pragma unroll
        for (int z = 0; z < W; z++) acc[c][z] = zero;
      since = 0;
    }
#pragma unroll 2
    for (int i = 0; i < nb; i++) {
      const int pk = s_o[i];
      const int slab = (pk >> 16) / TL;
      if (slab != zslab) {
        if (zslab >= 0) {
          const int steps = slab - zslab;
          if (steps * TL >= W) {
            commit(zslab * TL, 0, W);
#pragma unroll
            for (int c = 0; c < 2; c++)
#pragma unroll
              for (int z = 0; z < W; z++) acc[c][z] = zero;
          } else {
            for (int q = 0; q < steps; q++) {
              commit((zslab + q) * TL, 0, TL);
#pragma unroll
              for (int c = 0; c < 2; c++) {
#pragma unroll
                for (int z = 0; z < W - TL; z++) acc[c][z] = acc[c][z + TL];
#pragma unroll
                for (int z = W - TL; z < W; z++) acc[c][z] = zero;
              }
            }
          }
        }
        zslab = slab;
        since = 0;
      }
      since++;
      if (FONLY) {
        const T *w = s_w[i];
        const C zero2 = {(T)0, (T)0};
        const C fa = active ? ((const C *)(w + WP))[ca] : zero2;
        const T py0 = w[WP + 2 * R4 + cb], py1 = w[WP + 2 * R4 + cb + HR];
        T pz[WP];
        load_row<WP>(w, pz);
        const T h0r = fa.x * py0, h0i = fa.y * py0, h1r = fa.x * py1, h1i = fa.y * py1;
#pragma unroll
        for (int z = 0; z < W; z++) {
          acc_fma(acc[0][z], h0r, h0i, pz[z]);
          acc_fma(acc[1][z], h1r, h1i, pz[z]);
        }
        continue;
      }
      const int da = ca - (pk & 0xff), o1 = (pk >> 8) & 0xff;
      const bool row = active && (unsigned)da < (unsigned)CUT;
      const bool cov0 = row && (unsigned)(cb - o1) < (unsigned)CUT;
      const bool cov1 = row && (unsigned)(cb + HR - o1) < (unsigned)CUT;
      if (cov0 || cov1) {
        const T *w = s_w[i];
        const T px = w[WP + da];
        T fr = 0, fi = 0, g0r = 0, g0i = 0, g1r = 0, g1i = 0, g2r = 0, g2i = 0, dpx = 0;
        if (DF) {
          fr = px * s_v[i][0];
          fi = px * s_v[i][1];
        }
        if (DG) {
          dpx = w[WREC + WP + da];
          g0r = dpx * s_v[i][2];
          g0i = dpx * s_v[i][3];
          g1r = px * s_v[i][4];
          g1i = px * s_v[i][5];
          g2r = px * s_v[i][6];
          g2i = px * s_v[i][7];
        }
        T pz[WP];
        load_row<WP>(w, pz);
        T dz[DG ? WP : 1];
        if (DG) load_row<WP>(w + WREC, dz);
#pragma unroll
        for (int c = 0; c < 2; c++) {
          const bool cov = c ? cov1 : cov0;
          if (cov) {
            const int db = cb + c * HR - ((pk >> 8) & 0xff);
            const T py = w[WP + CP + db];
            // h1 multiplies psi_z, h2 multiplies psi_z'
            T h1r = fr * py, h1i = fi * py;
            if (DG) {
              const T dpy = w[WREC + WP + CP + db];
              h1r += g0r * py + g1r * dpy;
              h1i += g0i * py + g1i * dpy;
            }
#pragma unroll
            for (int z = 0; z < W; z++) acc_fma(acc[c][z], h1r, h1i, pz[z]);
            if (DG) {
              const T h2r = g2r * py, h2i = g2i * py;
#pragma unroll
              for (int z = 0; z < W; z++) acc_fma(acc[c][z], h2r, h2i, dz[z]);
            }
          }
        }
      }
    }
  }
  // --- commit the last window -----------------------------------------------------
  if (!active || zslab < 0) return;
  commit(zslab * TL, 0, W);
}

template <typename T, int CUT, int MODE>
static void run_spread_line(const ConvArgs &a, cudaStream_t s) {
  k_spread_line<T, CUT, MODE><<<a.bin.max_subs, LineGeom<CUT>::THREADS, 0, s>>>(a);
}

template <typename T, int MODE>
static bool spread_line_by_cut(const ConvArgs &a, cudaStream_t s) {
  switch (a.w.cut) {
    case 5: run_spread_line<T, 5, MODE>(a, s); return true;
    case 7: run_spread_line<T, 7, MODE>(a, s); return true;
    case 9: run_spread_line<T, 9, MODE>(a, s); return true;
    case 11: run_spread_line<T, 11, MODE>(a, s); return true;
    case 13: run_spread_line<T, 13, MODE>(a, s); return true;
    case 15: run_spread_line<T, 15, MODE>(a, s); return true;
    default: return false;
  }
}

template <typename T>
static bool spread_line_t(const ConvArgs &a, int mode, cudaStream_t s) {
  switch (mode) {
    case 1: return spread_line_by_cut<T, 1>(a, s);
    case 2: return spread_line_by_cut<T, 2>(a, s);
    case 3: return spread_line_by_cut<T, 3>(a, s);
    default: return false;
  }
}

}  // namespace pg
