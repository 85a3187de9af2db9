// interp_tile.cuh -- interpolation B with one warp per node over a
// shared-memory copy of the tile's region; instantiated per precision in
// interp_tile_f32.cu and interp_tile_f64.cu.
//
// Reference: loop_over_particles_trafo (kernel/ndft-parallel.c:2703-2888)
// with the interpolation loops of kernel/assign.c:667-1159.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include "pg_conv.cuh"
#include "pg_kernels.h"
#include "pg_math.cuh"

namespace pg {

// ---------------------------------------------------------------------------
// interpolation B, tiled.  The CTA stages its tile's (TE+2m)^3 region in
// shared memory (TE = 4: a tile of a line binning, whose records carry the
// full lowest z index; TE = 8: an 8x8x8-cell tile binning), then walks its
// nodes in batches: (1) all threads evaluate
// the window values of the batch (3 x cutoff per node and derivative), (2)
// one warp per node sums the 13^3 stencil -- lanes (row = lane/16, col =
// lane%16) read two z-rows of 13 consecutive grid values per step, with the
// x-window in registers -- and reduces with shuffles, (3) the batch's results
// are converted and written by all threads.
// ---------------------------------------------------------------------------
template <typename T, int CUT, int MODE, int TE>
struct InterpGeom {
  static constexpr bool DF = (MODE & 1) != 0, DG = (MODE & 2) != 0, DH = (MODE & 4) != 0;
  static constexpr int NDER = DH ? 2 : (DG ? 1 : 0);
  static constexpr int R = TE + CUT - 1, PL = R * R, VOL = R * R * R;
  static constexpr int NV = 3 * CUT * (NDER + 1);
  static constexpr int NC = (DF ? 1 : 0) + (DG ? 3 : 0) + (DH ? 6 : 0);
  static constexpr int NBI = sizeof(T) == 4 ? 48 : 32;
  static constexpr size_t SMEM = (size_t)VOL * 2 * sizeof(T) + (size_t)NBI * (NV + 2 * NC + 4) * sizeof(T) +
                                 (size_t)NBI * 2 * sizeof(int);
};

template <typename T, int CUT, int MODE, int TE>
__global__ void __launch_bounds__(256) k_interp_tile(ConvArgs a) {
  typedef typename Cplx<T>::type C;
  typedef InterpGeom<T, CUT, MODE, TE> G;
  constexpr bool DF = G::DF, DG = G::DG, DH = G::DH;
  constexpr int NDER = G::NDER, R = G::R, PL = G::PL, VOL = G::VOL, NV = G::NV, NC = G::NC, NBI = G::NBI;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *reg = (C *)smem_raw;
  T *s_w = (T *)(reg + VOL);     // [NBI][NV]
  T *s_res = s_w + NBI * NV;     // [NBI][2*NC]
  T *s_d = s_res + NBI * 2 * NC; // [NBI][4]
  int *s_j = (int *)(s_d + NBI * 4);
  int *s_o = s_j + NBI;
  const Binning &b = a.bin;
  const int sub = blockIdx.x;
  if (sub >= *b.nsub) return;
  const int tile = b.sub_tile[sub], first = b.sub_first[sub], cnt = b.sub_cnt[sub];
  if (cnt <= 0) return;  // an empty tile of an ordered sub-problem list
  int base[3];
  tile_base(b, tile, base);
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  const int tid = threadIdx.x;
  const C *grid = (const C *)a.grid;
  load_region<R>(reg, grid, base, n0, n1, n2, a.real_only);
  const int lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  const int row = lane >> 4, col = lane & 15;
  const T scale = a.use_il ? (T)0.5 : (T)1;
  for (int b0 = 0; b0 < cnt; b0 += NBI) {
    const int nb = min(NBI, cnt - b0);
    __syncthreads();  // region loaded / previous batch flushed
    for (int i = tid; i < nb; i += blockDim.x) {
      T d[3];
      int pk;
      load_rec_raw(b.rec, first + b0 + i, d, &pk);
      s_d[4 * i] = d[0];
      s_d[4 * i + 1] = d[1];
      s_d[4 * i + 2] = d[2];
      s_o[i] = pk;
      s_j[i] = b.perm[first + b0 + i];
    }
    __syncthreads();
    // node-fastest: a warp shares one (axis, stencil point), so the fitted
    // polynomial rows are broadcast loads
#pragma unroll 2  // two independent polynomial chains per thread
    for (int v = tid; v < NBI * 3 * CUT; v += blockDim.x) {
      const int e = v / NBI, i = v - e * NBI;
      if (i >= nb) continue;
      const int t = e / CUT, sidx = e - t * CUT;
      T out[3];
      window_point<T>(a.w, t, sidx, s_d[4 * i + t], NDER, out);
      T *wv = s_w + i * NV;
      wv[e] = out[0];
      if (NDER >= 1) wv[3 * CUT + e] = out[1];
      if (NDER >= 2) wv[6 * CUT + e] = out[2];
    }
    __syncthreads();
    for (int i = warp; i < nb; i += nwarp) {
      const T *wv = s_w + i * NV;
      int o[3];
      unpack_corner(s_o[i], o);
      if (TE == 4) o[2] = ((s_o[i] >> 16) & 0x7fff) - base[2];  // line records: the full u2
      T px[CUT], dpx[CUT], ddpx[CUT];
#pragma unroll
      for (int l = 0; l < CUT; l++) {
        px[l] = wv[l];
        if (NDER >= 1) dpx[l] = wv[3 * CUT + l];
        if (NDER >= 2) ddpx[l] = wv[6 * CUT + l];
      }
      const C zero = {(T)0, (T)0};
      C af = zero, ag[3] = {zero, zero, zero}, ah[6] = {zero, zero, zero, zero, zero, zero};
      if (col < CUT) {
        const T pz = wv[2 * CUT + col];
        const T dz = (NDER >= 1) ? wv[3 * CUT + 2 * CUT + col] : (T)0;
        const T ddz = (NDER >= 2) ? wv[6 * CUT + 2 * CUT + col] : (T)0;
        const C *pc = reg + (o[0] * R + o[1]) * R + (o[2] + col);
#pragma unroll
        for (int it = 0; it < (CUT + 1) / 2; it++) {
          const int l1 = 2 * it + row;
          if (l1 < CUT) {
            const T py = wv[CUT + l1];
            const T dy = (NDER >= 1) ? wv[3 * CUT + CUT + l1] : (T)0;
            const T ddy = (NDER >= 2) ? wv[6 * CUT + CUT + l1] : (T)0;
            const C *p = pc + l1 * R;
            // even and odd x planes in separate chains (independent FMAs),
            // added at the end of the row
            C sxp[2] = {zero, zero}, sdp[2] = {zero, zero}, sddp[2] = {zero, zero};
#pragma unroll
            for (int l0 = 0; l0 < CUT; l0++) {
              const C g = p[l0 * PL];
              cfma(sxp[l0 & 1], px[l0], g);
              if (NDER >= 1) cfma(sdp[l0 & 1], dpx[l0], g);
              if (NDER >= 2) cfma(sddp[l0 & 1], ddpx[l0], g);
            }
            const C sx = cadd(sxp[0], sxp[1]);
            const C sd = NDER >= 1 ? cadd(sdp[0], sdp[1]) : zero;
            const C sdd = NDER >= 2 ? cadd(sddp[0], sddp[1]) : zero;
            const T wyz = py * pz;
            if (DF) cfma(af, wyz, sx);
            if (DG) {
              cfma(ag[0], wyz, sd);
              cfma(ag[1], dy * pz, sx);
              cfma(ag[2], py * dz, sx);
            }
            if (DH) {
              cfma(ah[0], wyz, sdd);
              cfma(ah[1], dy * pz, sd);
              cfma(ah[2], py * dz, sd);
              cfma(ah[3], ddy * pz, sx);
              cfma(ah[4], dy * dz, sx);
              cfma(ah[5], py * ddz, sx);
            }
          }
        }
      }
      T *res = s_res + i * 2 * NC;
      int c = 0;
      if (DF) {
        T r = warp_sum(af.x), im = warp_sum(af.y);
        if (lane == 0) {
          res[0] = r * scale;
          res[1] = im * scale;
        }
        c = 1;
      }
      if (DG) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          T r = warp_sum(ag[k].x), im = warp_sum(ag[k].y);
          if (lane == 0) {
            res[2 * (c + k)] = r * scale;
            res[2 * (c + k) + 1] = im * scale;
          }
        }
      }
      if (DH) {
#pragma unroll
        for (int k = 0; k < 6; k++) {
          T r = warp_sum(ah[k].x), im = warp_sum(ah[k].y);
          if (lane == 0) {
            res[2 * k] = r * scale;
            res[2 * k + 1] = im * scale;
          }
        }
      }
    }
    __syncthreads();
    // write the batch: one thread per (node, output component)
    for (int v = tid; v < nb * NC; v += blockDim.x) {
      const int i = v / NC, k = v - i * NC;
      const int64_t ind = (int64_t)s_j[i] * a.stride + a.offset;
      double *out;
      int64_t e;
      if (DH) {
        out = a.hess_out;
        e = 6 * ind + k;
      } else if (DF && k == 0) {
        out = a.f_out;
        e = ind;
      } else {
        out = a.grad_out;
        e = 3 * ind + (k - (DF ? 1 : 0));
      }
      const double vr = (double)s_res[i * 2 * NC + 2 * k], vi = (double)s_res[i * 2 * NC + 2 * k + 1];
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
}

template <typename T, int CUT, int MODE, int TE>
static void run_interp_tile(const ConvArgs &a, cudaStream_t s) {
  const size_t sm = InterpGeom<T, CUT, MODE, TE>::SMEM;
  // the shared-memory opt-in is a per-device attribute of the kernel
  static std::atomic<unsigned long long> attr_done{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(attr_done.load() & bit)) {
    cudaFuncSetAttribute(k_interp_tile<T, CUT, MODE, TE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr_done.fetch_or(bit);
  }
  k_interp_tile<T, CUT, MODE, TE><<<a.bin.max_subs, 256, sm, s>>>(a);
}

template <typename T, int MODE, int TE>
static bool interp_tile_by_cut(const ConvArgs &a, cudaStream_t s) {
  switch (a.w.cut) {
    case 5: run_interp_tile<T, 5, MODE, TE>(a, s); return true;
    case 7: run_interp_tile<T, 7, MODE, TE>(a, s); return true;
    case 9: run_interp_tile<T, 9, MODE, TE>(a, s); return true;
    case 11: run_interp_tile<T, 11, MODE, TE>(a, s); return true;
    case 13: run_interp_tile<T, 13, MODE, TE>(a, s); return true;
    case 15: run_interp_tile<T, 15, MODE, TE>(a, s); return true;
    default: return false;
  }
}

// 4x4x4 tiles of a line binning in every mode; 8x8x8 tiles for the
// FP32-mixed plans (conv methods 2 and 3)
template <typename T>
static bool interp_tile_t(const ConvArgs &a, int mode, cudaStream_t s) {
  if (a.bin.T[0] == 8) {
    if (sizeof(T) != 4) return false;
    switch (mode) {
      case 1: return interp_tile_by_cut<T, 1, 8>(a, s);
      case 2: return interp_tile_by_cut<T, 2, 8>(a, s);
      case 3: return interp_tile_by_cut<T, 3, 8>(a, s);
      case 4: return interp_tile_by_cut<T, 4, 8>(a, s);
      default: return false;
    }
  }
  if (a.bin.T[0] != 4) return false;
  switch (mode) {
    case 1: return interp_tile_by_cut<T, 1, 4>(a, s);
    case 2: return interp_tile_by_cut<T, 2, 4>(a, s);
    case 3: return interp_tile_by_cut<T, 3, 4>(a, s);
    case 4: return interp_tile_by_cut<T, 4, 4>(a, s);
    default: return false;
  }
}

}  // namespace pg
