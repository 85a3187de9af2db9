// conv.cu -- the convolution with the window: interpolation B (grid -> nodes,
// pnfft_trafo) and spreading B^T (nodes -> grid, pnfft_adj), plus the binning
// of nodes onto grid tiles that both use.
//
// Reference: loop_over_particles_trafo / _adj (kernel/ndft-parallel.c:2703-3009)
// with the stencil loops of kernel/assign.c:478-1159.  The reference walks the
// nodes one by one over a ghost-celled local grid; here
//   * nodes are binned by the tile that holds their lowest stencil point
//     (floor(n x) - m, wrapped mod n), with a counting sort;
//   * one CTA takes one run of <= sub_max nodes of one tile, stages the tile
//     plus its (2m) halo in shared memory, and one warp handles one node:
//     lanes (row = lane/16, col = lane%16) cover two z-rows of the 13x13x13
//     stencil per step, so every half-warp reads 13 consecutive grid values;
//   * B reduces the per-lane partial sums with warp shuffles; B^T adds into
//     the shared tile with shared-memory atomics and commits the tile with
//     one global atomic per touched grid point;
//   * the periodic ghost-cell exchange/reduce of the reference
//     (ndft-parallel.c:2558, 2679) becomes the modulo wrap of the tile loads
//     and commits.
// Window values are evaluated per node in registers/shared memory
// (pg_math.cuh) or read from the PNFFT_PRE_*_PSI interpolation tables.
#include <cuda_runtime.h>
#include <stdio.h>

#include "pg_kernels.h"
#include "pg_math.cuh"

namespace pg {

template <typename T>
struct Cplx;
template <>
struct Cplx<float> {
  typedef float2 type;
};
template <>
struct Cplx<double> {
  typedef double2 type;
};

// ---------------------------------------------------------------------------
// node -> grid index, bit-exact with ndft-parallel.c:2732-2753, 2165-2174:
// x' = x (+ 0.5/n when interlaced), fnx = floor(n x'), u = fnx - m, then the
// fold x' -= 1 (fnx -= n) when x' >= 0.5.  Explicit _rn intrinsics keep nvcc
// from fusing the operations into an FMA.
// ---------------------------------------------------------------------------
struct AxisPos {
  double dist;  // n x' - fnx after the fold, in [0,1)
  int u;        // lowest stencil index wrapped into [0, n)
};

__device__ __forceinline__ AxisPos axis_pos(double x, int n, int m, int il) {
  double xs = x;
  if (il) xs = __dadd_rn(xs, __ddiv_rn(0.5, (double)n));
  double fnx = floor(__dmul_rn((double)n, xs));
  long long u = (long long)fnx - m;
  if (il && xs >= 0.5) {
    xs = __dsub_rn(xs, 1.0);
    fnx -= (double)n;
  }
  AxisPos p;
  p.dist = __dsub_rn(__dmul_rn((double)n, xs), fnx);
  long long w = u % n;
  if (w < 0) w += n;
  p.u = (int)w;
  return p;
}

// window values of one node: ws[der*3*cut + t*cut + s]
template <typename T>
__device__ __forceinline__ void warp_windows(const WindowArgs &w, const double *dist, int nder, T *ws, int lane) {
  const int cut = w.cut;
  for (int e = lane; e < 3 * cut; e += 32) {
    int t = e / cut, s = e - t * cut;
    T out[3] = {(T)0, (T)0, (T)0};
    if (w.intpol_order >= 0) {
      double dK = dist[t] * (double)w.intpol_K;
      long long k = (long long)floor(dK);
      T dk = (T)(dK - (double)k);
      size_t base = ((size_t)k * cut + s) * (size_t)(w.intpol_order + 1);
      for (int d = 0; d <= nder; d++) out[d] = intpol<T>(w.intpol_order, (const T *)w.tab[d][t] + base, dk);
    } else {
      T y = (T)dist[t] + (T)(w.m - s);
      T smd = (T)s - (T)dist[t];
      window_eval<T>(w.kind, w.m, (T)w.n[t], (T)w.b[t], y, smd, nder, out);
    }
    ws[e] = out[0];
    if (nder >= 1) ws[3 * cut + e] = out[1];
    if (nder >= 2) ws[6 * cut + e] = out[2];
  }
}

// ---------------------------------------------------------------------------
// binning
// ---------------------------------------------------------------------------
__global__ void k_bin_keys(const double *__restrict__ x, int64_t M, int n0, int n1, int n2, int m, int il, int T0,
                           int T1, int T2, int nt1, int nt2, int *__restrict__ key, int *__restrict__ count) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  AxisPos p0 = axis_pos(x[3 * j + 0], n0, m, il);
  AxisPos p1 = axis_pos(x[3 * j + 1], n1, m, il);
  AxisPos p2 = axis_pos(x[3 * j + 2], n2, m, il);
  int tile = ((p0.u / T0) * nt1 + p1.u / T1) * nt2 + p2.u / T2;
  key[j] = tile;
  atomicAdd(&count[tile], 1);
}

// exclusive scans of count and of the number of sub-problems per tile (one CTA)
__global__ void __launch_bounds__(1024) k_bin_scan(Binning b) {
  __shared__ int s_a[1024], s_b[1024];
  const int tid = threadIdx.x, nt = b.ntiles;
  const int chunk = (nt + 1023) / 1024;
  const int lo = min(nt, tid * chunk), hi = min(nt, lo + chunk);
  int sa = 0, sb = 0;
  for (int i = lo; i < hi; i++) {
    int c = b.count[i];
    sa += c;
    sb += (c + b.sub_max - 1) / b.sub_max;
  }
  s_a[tid] = sa;
  s_b[tid] = sb;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    int va = (tid >= off) ? s_a[tid - off] : 0;
    int vb = (tid >= off) ? s_b[tid - off] : 0;
    __syncthreads();
    s_a[tid] += va;
    s_b[tid] += vb;
    __syncthreads();
  }
  int pa = s_a[tid] - sa, pb = s_b[tid] - sb;
  for (int i = lo; i < hi; i++) {
    int c = b.count[i];
    int ns = (c + b.sub_max - 1) / b.sub_max;
    b.start[i] = pa;
    b.cursor[i] = 0;
    b.nsub_tile[i] = ns;
    b.sub_off[i] = pb;
    pa += c;
    pb += ns;
  }
  if (tid == 1023) *b.nsub = s_b[1023];
}

__global__ void k_bin_scatter(int64_t M, Binning b) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  int t = b.key[j];
  int pos = b.start[t] + atomicAdd(&b.cursor[t], 1);
  b.perm[pos] = (int)j;
}

__global__ void k_bin_subs(Binning b) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.ntiles) return;
  int ns = b.nsub_tile[t], off = b.sub_off[t], st = b.start[t], c = b.count[t];
  for (int i = 0; i < ns; i++) {
    b.sub_tile[off + i] = t;
    b.sub_first[off + i] = st + i * b.sub_max;
    b.sub_cnt[off + i] = min(b.sub_max, c - i * b.sub_max);
  }
}

void bin_nodes(const ConvArgs &a, cudaStream_t s) {
  const Binning &b = a.bin;
  cudaMemsetAsync(b.count, 0, sizeof(int) * b.ntiles, s);
  if (a.M > 0) {
    int th = 256;
    int64_t bl = (a.M + th - 1) / th;
    k_bin_keys<<<(unsigned)bl, th, 0, s>>>(a.x, a.M, a.w.n[0], a.w.n[1], a.w.n[2], a.w.m, a.il, b.T[0], b.T[1], b.T[2],
                                            b.ntile[1], b.ntile[2], b.key, b.count);
  }
  k_bin_scan<<<1, 1024, 0, s>>>(b);
  if (a.M > 0) {
    int th = 256;
    int64_t bl = (a.M + th - 1) / th;
    k_bin_scatter<<<(unsigned)bl, th, 0, s>>>(a.M, b);
  }
  k_bin_subs<<<(b.ntiles + 255) / 256, 256, 0, s>>>(b);
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void tile_base(const Binning &b, int tile, int *base) {
  int t2 = tile % b.ntile[2];
  int r = tile / b.ntile[2];
  int t1 = r % b.ntile[1];
  int t0 = r / b.ntile[1];
  base[0] = t0 * b.T[0];
  base[1] = t1 * b.T[1];
  base[2] = t2 * b.T[2];
}

__device__ __forceinline__ void atomic_add_grid(float2 *p, float2 v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_grid(double2 *p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

// ---------------------------------------------------------------------------
// interpolation B, tiled (compile-time cutoff CUT <= 16)
// ---------------------------------------------------------------------------
template <typename T, int CUT, int MODE>
__global__ void __launch_bounds__(256) k_interp_tile(ConvArgs a) {
  typedef typename Cplx<T>::type C;
  constexpr bool DF = (MODE & 1) != 0, DG = (MODE & 2) != 0, DH = (MODE & 4) != 0;
  constexpr int NDER = DH ? 2 : (DG ? 1 : 0);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Binning &b = a.bin;
  const int sub = blockIdx.x;
  if (sub >= *b.nsub) return;
  const int tile = b.sub_tile[sub], first = b.sub_first[sub], cnt = b.sub_cnt[sub];
  int base[3];
  tile_base(b, tile, base);
  const int R0 = b.T[0] + CUT - 1, R1 = b.T[1] + CUT - 1, R2 = b.T[2] + CUT - 1;
  const int vol = R0 * R1 * R2;
  C *reg = (C *)smem_raw;
  T *wsall = (T *)(reg + vol);
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  const C *grid = (const C *)a.grid;
  for (int i = threadIdx.x; i < vol; i += blockDim.x) {
    int c = i % R2, q = i / R2;
    int bb = q % R1, aa = q / R1;
    int g0 = (base[0] + aa) % n0, g1 = (base[1] + bb) % n1, g2 = (base[2] + c) % n2;
    C v = grid[((size_t)g0 * n1 + g1) * n2 + g2];
    if (a.real_only) v.y = (T)0;
    reg[i] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  T *ws = wsall + warp * (9 * CUT);
  const int row = lane >> 4, col = lane & 15;
  const T scale = a.use_il ? (T)0.5 : (T)1;
  for (int q = warp; q < cnt; q += nwarp) {
    const int j = b.perm[first + q];
    double dist[3];
    int o[3];
#pragma unroll
    for (int t = 0; t < 3; t++) {
      AxisPos p = axis_pos(a.x[3 * (int64_t)j + t], a.w.n[t], a.w.m, a.il);
      dist[t] = p.dist;
      o[t] = p.u - base[t];
    }
    warp_windows<T>(a.w, dist, NDER, ws, lane);
    __syncwarp();
    T px[CUT], dpx[CUT], ddpx[CUT];
#pragma unroll
    for (int l = 0; l < CUT; l++) {
      px[l] = ws[l];
      if (NDER >= 1) dpx[l] = ws[3 * CUT + l];
      if (NDER >= 2) ddpx[l] = ws[6 * CUT + l];
    }
    // accumulators: f; grad x,y,z; hessian xx,xy,xz,yy,yz,zz
    T af_r = 0, af_i = 0;
    T ag_r[3] = {0, 0, 0}, ag_i[3] = {0, 0, 0};
    T ah_r[6] = {0, 0, 0, 0, 0, 0}, ah_i[6] = {0, 0, 0, 0, 0, 0};
    if (col < CUT) {
      const T pz = ws[2 * CUT + col];
      const T dz = (NDER >= 1) ? ws[3 * CUT + 2 * CUT + col] : (T)0;
      const T ddz = (NDER >= 2) ? ws[6 * CUT + 2 * CUT + col] : (T)0;
      for (int l1 = row; l1 < CUT; l1 += 2) {
        const T py = ws[CUT + l1];
        const T dy = (NDER >= 1) ? ws[3 * CUT + CUT + l1] : (T)0;
        const T ddy = (NDER >= 2) ? ws[6 * CUT + CUT + l1] : (T)0;
        const C *p = reg + ((size_t)o[0] * R1 + (o[1] + l1)) * R2 + (o[2] + col);
        T s_r = 0, s_i = 0, sd_r = 0, sd_i = 0, sdd_r = 0, sdd_i = 0;
#pragma unroll
        for (int l0 = 0; l0 < CUT; l0++) {
          C g = p[(size_t)l0 * R1 * R2];
          s_r += px[l0] * g.x;
          s_i += px[l0] * g.y;
          if (NDER >= 1) {
            sd_r += dpx[l0] * g.x;
            sd_i += dpx[l0] * g.y;
          }
          if (NDER >= 2) {
            sdd_r += ddpx[l0] * g.x;
            sdd_i += ddpx[l0] * g.y;
          }
        }
        const T wyz = py * pz;
        if (DF) {
          af_r += wyz * s_r;
          af_i += wyz * s_i;
        }
        if (DG) {
          ag_r[0] += wyz * sd_r;
          ag_i[0] += wyz * sd_i;
          ag_r[1] += dy * pz * s_r;
          ag_i[1] += dy * pz * s_i;
          ag_r[2] += py * dz * s_r;
          ag_i[2] += py * dz * s_i;
        }
        if (DH) {
          ah_r[0] += wyz * sdd_r;
          ah_i[0] += wyz * sdd_i;
          ah_r[1] += dy * pz * sd_r;
          ah_i[1] += dy * pz * sd_i;
          ah_r[2] += py * dz * sd_r;
          ah_i[2] += py * dz * sd_i;
          ah_r[3] += ddy * pz * s_r;
          ah_i[3] += ddy * pz * s_i;
          ah_r[4] += dy * dz * s_r;
          ah_i[4] += dy * dz * s_i;
          ah_r[5] += py * ddz * s_r;
          ah_i[5] += py * ddz * s_i;
        }
      }
    }
    const int64_t ind = (int64_t)j * a.stride + a.offset;
    if (DF) {
      af_r = warp_sum(af_r);
      af_i = warp_sum(af_i);
      if (lane == 0) {
        if (a.real_io) a.f_out[ind] += (double)(af_r * scale);
        else {
          a.f_out[2 * ind] += (double)(af_r * scale);
          a.f_out[2 * ind + 1] += (double)(af_i * scale);
        }
      }
    }
    if (DG) {
#pragma unroll
      for (int c = 0; c < 3; c++) {
        T r = warp_sum(ag_r[c]), im = warp_sum(ag_i[c]);
        if (lane == 0) {
          if (a.real_io) a.grad_out[3 * ind + c] += (double)(r * scale);
          else {
            a.grad_out[2 * (3 * ind + c)] += (double)(r * scale);
            a.grad_out[2 * (3 * ind + c) + 1] += (double)(im * scale);
          }
        }
      }
    }
    if (DH) {
#pragma unroll
      for (int c = 0; c < 6; c++) {
        T r = warp_sum(ah_r[c]), im = warp_sum(ah_i[c]);
        if (lane == 0) {
          if (a.real_io) a.hess_out[6 * ind + c] += (double)(r * scale);
          else {
            a.hess_out[2 * (6 * ind + c)] += (double)(r * scale);
            a.hess_out[2 * (6 * ind + c) + 1] += (double)(im * scale);
          }
        }
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// spreading B^T, tiled (compile-time cutoff CUT <= 16)
// ---------------------------------------------------------------------------
template <typename T, int CUT, int MODE>
__global__ void __launch_bounds__(256) k_spread_tile(ConvArgs a) {
  typedef typename Cplx<T>::type C;
  constexpr bool DF = (MODE & 1) != 0, DG = (MODE & 2) != 0;
  constexpr int NDER = DG ? 1 : 0;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Binning &b = a.bin;
  const int sub = blockIdx.x;
  if (sub >= *b.nsub) return;
  const int tile = b.sub_tile[sub], first = b.sub_first[sub], cnt = b.sub_cnt[sub];
  int base[3];
  tile_base(b, tile, base);
  const int R0 = b.T[0] + CUT - 1, R1 = b.T[1] + CUT - 1, R2 = b.T[2] + CUT - 1;
  const int vol = R0 * R1 * R2;
  T *sre = (T *)smem_raw;
  T *sim = sre + vol;
  T *wsall = sim + vol;
  for (int i = threadIdx.x; i < vol; i += blockDim.x) {
    sre[i] = (T)0;
    sim[i] = (T)0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  T *ws = wsall + warp * (6 * CUT);
  const int row = lane >> 4, col = lane & 15;
  const T scale = a.use_il ? (T)0.5 : (T)1;
  for (int q = warp; q < cnt; q += nwarp) {
    const int j = b.perm[first + q];
    double dist[3];
    int o[3];
#pragma unroll
    for (int t = 0; t < 3; t++) {
      AxisPos p = axis_pos(a.x[3 * (int64_t)j + t], a.w.n[t], a.w.m, a.il);
      dist[t] = p.dist;
      o[t] = p.u - base[t];
    }
    warp_windows<T>(a.w, dist, NDER, ws, lane);
    const int64_t ind = (int64_t)j * a.stride + a.offset;
    T f_r = 0, f_i = 0;
    T g_r[3] = {0, 0, 0}, g_i[3] = {0, 0, 0};
    if (DF) {
      if (a.real_io) f_r = (T)a.f_in[ind];
      else {
        f_r = (T)a.f_in[2 * ind];
        f_i = (T)a.f_in[2 * ind + 1];
      }
      f_r *= scale;
      f_i *= scale;
    }
    if (DG) {
#pragma unroll
      for (int c = 0; c < 3; c++) {
        if (a.real_io) g_r[c] = (T)a.grad_in[3 * ind + c];
        else {
          g_r[c] = (T)a.grad_in[2 * (3 * ind + c)];
          g_i[c] = (T)a.grad_in[2 * (3 * ind + c) + 1];
        }
        g_r[c] *= scale;
        g_i[c] *= scale;
      }
    }
    __syncwarp();
    T px[CUT], dpx[CUT];
#pragma unroll
    for (int l = 0; l < CUT; l++) {
      px[l] = ws[l];
      if (DG) dpx[l] = ws[3 * CUT + l];
    }
    if (col < CUT) {
      const T pz = ws[2 * CUT + col];
      const T dz = DG ? ws[3 * CUT + 2 * CUT + col] : (T)0;
      for (int l1 = row; l1 < CUT; l1 += 2) {
        const T py = ws[CUT + l1];
        const T dy = DG ? ws[3 * CUT + CUT + l1] : (T)0;
        // w(l0) = px[l0] * c1 + dpx[l0] * c2
        T c1_r = 0, c1_i = 0, c2_r = 0, c2_i = 0;
        if (DF) {
          c1_r = py * pz * f_r;
          c1_i = py * pz * f_i;
        }
        if (DG) {
          c1_r += dy * pz * g_r[1] + py * dz * g_r[2];
          c1_i += dy * pz * g_i[1] + py * dz * g_i[2];
          c2_r = py * pz * g_r[0];
          c2_i = py * pz * g_i[0];
        }
        const int rb = ((o[0]) * R1 + (o[1] + l1)) * R2 + (o[2] + col);
#pragma unroll
        for (int l0 = 0; l0 < CUT; l0++) {
          T wr = px[l0] * c1_r, wi = px[l0] * c1_i;
          if (DG) {
            wr += dpx[l0] * c2_r;
            wi += dpx[l0] * c2_i;
          }
          atomicAdd(&sre[rb + l0 * R1 * R2], wr);
          atomicAdd(&sim[rb + l0 * R1 * R2], wi);
        }
      }
    }
    __syncwarp();
  }
  __syncthreads();
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  C *grid = (C *)a.grid;
  for (int i = threadIdx.x; i < vol; i += blockDim.x) {
    C v;
    v.x = sre[i];
    v.y = sim[i];
    if (v.x == (T)0 && v.y == (T)0) continue;
    int c = i % R2, q = i / R2;
    int bb = q % R1, aa = q / R1;
    int g0 = (base[0] + aa) % n0, g1 = (base[1] + bb) % n1, g2 = (base[2] + c) % n2;
    atomic_add_grid(&grid[((size_t)g0 * n1 + g1) * n2 + g2], v);
  }
}

// ---------------------------------------------------------------------------
// generic kernels for any cutoff: one thread per node, global memory
// ---------------------------------------------------------------------------
template <typename T, int MODE>
__global__ void k_interp_generic(ConvArgs a) {
  typedef typename Cplx<T>::type C;
  constexpr bool DF = (MODE & 1) != 0, DG = (MODE & 2) != 0, DH = (MODE & 4) != 0;
  constexpr int NDER = DH ? 2 : (DG ? 1 : 0);
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.M) return;
  const int j = a.bin.perm[q];
  const int cut = a.w.cut;
  T ws[9 * 64];
  double dist[3];
  int u[3];
  for (int t = 0; t < 3; t++) {
    AxisPos p = axis_pos(a.x[3 * (int64_t)j + t], a.w.n[t], a.w.m, a.il);
    dist[t] = p.dist;
    u[t] = p.u;
  }
  // single-thread window evaluation: reuse warp_windows with a 1-lane stride
  for (int e = 0; e < 3 * cut; e++) {
    int t = e / cut, s = e - t * cut;
    T out[3] = {(T)0, (T)0, (T)0};
    if (a.w.intpol_order >= 0) {
      double dK = dist[t] * (double)a.w.intpol_K;
      long long k = (long long)floor(dK);
      T dk = (T)(dK - (double)k);
      size_t bse = ((size_t)k * cut + s) * (size_t)(a.w.intpol_order + 1);
      for (int d = 0; d <= NDER; d++) out[d] = intpol<T>(a.w.intpol_order, (const T *)a.w.tab[d][t] + bse, dk);
    } else {
      window_eval<T>(a.w.kind, a.w.m, (T)a.w.n[t], (T)a.w.b[t], (T)dist[t] + (T)(a.w.m - s), (T)s - (T)dist[t], NDER,
                     out);
    }
    ws[e] = out[0];
    ws[3 * cut + e] = out[1];
    ws[6 * cut + e] = out[2];
  }
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  const C *grid = (const C *)a.grid;
  T af_r = 0, af_i = 0, ag_r[3] = {0, 0, 0}, ag_i[3] = {0, 0, 0}, ah_r[6] = {0}, ah_i[6] = {0};
  for (int l0 = 0; l0 < cut; l0++) {
    int g0 = (u[0] + l0) % n0;
    for (int l1 = 0; l1 < cut; l1++) {
      int g1 = (u[1] + l1) % n1;
      const T px = ws[l0], py = ws[cut + l1], dx = ws[3 * cut + l0], dy = ws[3 * cut + cut + l1];
      const T ddx = ws[6 * cut + l0], ddy = ws[6 * cut + cut + l1];
      for (int l2 = 0; l2 < cut; l2++) {
        int g2 = (u[2] + l2) % n2;
        C g = grid[((size_t)g0 * n1 + g1) * n2 + g2];
        if (a.real_only) g.y = (T)0;
        const T pz = ws[2 * cut + l2], dz = ws[3 * cut + 2 * cut + l2], ddz = ws[6 * cut + 2 * cut + l2];
        if (DF) {
          af_r += px * py * pz * g.x;
          af_i += px * py * pz * g.y;
        }
        if (DG) {
          T w0 = dx * py * pz, w1 = px * dy * pz, w2 = px * py * dz;
          ag_r[0] += w0 * g.x;
          ag_i[0] += w0 * g.y;
          ag_r[1] += w1 * g.x;
          ag_i[1] += w1 * g.y;
          ag_r[2] += w2 * g.x;
          ag_i[2] += w2 * g.y;
        }
        if (DH) {
          T w[6] = {ddx * py * pz, dx * dy * pz, dx * py * dz, px * ddy * pz, px * dy * dz, px * py * ddz};
          for (int c = 0; c < 6; c++) {
            ah_r[c] += w[c] * g.x;
            ah_i[c] += w[c] * g.y;
          }
        }
      }
    }
  }
  const T scale = a.use_il ? (T)0.5 : (T)1;
  const int64_t ind = (int64_t)j * a.stride + a.offset;
  if (DF) {
    if (a.real_io) a.f_out[ind] += (double)(af_r * scale);
    else {
      a.f_out[2 * ind] += (double)(af_r * scale);
      a.f_out[2 * ind + 1] += (double)(af_i * scale);
    }
  }
  if (DG)
    for (int c = 0; c < 3; c++) {
      if (a.real_io) a.grad_out[3 * ind + c] += (double)(ag_r[c] * scale);
      else {
        a.grad_out[2 * (3 * ind + c)] += (double)(ag_r[c] * scale);
        a.grad_out[2 * (3 * ind + c) + 1] += (double)(ag_i[c] * scale);
      }
    }
  if (DH)
    for (int c = 0; c < 6; c++) {
      if (a.real_io) a.hess_out[6 * ind + c] += (double)(ah_r[c] * scale);
      else {
        a.hess_out[2 * (6 * ind + c)] += (double)(ah_r[c] * scale);
        a.hess_out[2 * (6 * ind + c) + 1] += (double)(ah_i[c] * scale);
      }
    }
}

template <typename T, int MODE>
__global__ void k_spread_generic(ConvArgs a) {
  typedef typename Cplx<T>::type C;
  constexpr bool DF = (MODE & 1) != 0, DG = (MODE & 2) != 0;
  constexpr int NDER = DG ? 1 : 0;
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.M) return;
  const int j = a.bin.perm[q];
  const int cut = a.w.cut;
  T ws[6 * 64];
  double dist[3];
  int u[3];
  for (int t = 0; t < 3; t++) {
    AxisPos p = axis_pos(a.x[3 * (int64_t)j + t], a.w.n[t], a.w.m, a.il);
    dist[t] = p.dist;
    u[t] = p.u;
  }
  for (int e = 0; e < 3 * cut; e++) {
    int t = e / cut, s = e - t * cut;
    T out[3] = {(T)0, (T)0, (T)0};
    if (a.w.intpol_order >= 0) {
      double dK = dist[t] * (double)a.w.intpol_K;
      long long k = (long long)floor(dK);
      T dk = (T)(dK - (double)k);
      size_t bse = ((size_t)k * cut + s) * (size_t)(a.w.intpol_order + 1);
      for (int d = 0; d <= NDER; d++) out[d] = intpol<T>(a.w.intpol_order, (const T *)a.w.tab[d][t] + bse, dk);
    } else {
      window_eval<T>(a.w.kind, a.w.m, (T)a.w.n[t], (T)a.w.b[t], (T)dist[t] + (T)(a.w.m - s), (T)s - (T)dist[t], NDER,
                     out);
    }
    ws[e] = out[0];
    ws[3 * cut + e] = out[1];
  }
  const T scale = a.use_il ? (T)0.5 : (T)1;
  const int64_t ind = (int64_t)j * a.stride + a.offset;
  T f_r = 0, f_i = 0, g_r[3] = {0, 0, 0}, g_i[3] = {0, 0, 0};
  if (DF) {
    if (a.real_io) f_r = (T)a.f_in[ind];
    else {
      f_r = (T)a.f_in[2 * ind];
      f_i = (T)a.f_in[2 * ind + 1];
    }
  }
  if (DG)
    for (int c = 0; c < 3; c++) {
      if (a.real_io) g_r[c] = (T)a.grad_in[3 * ind + c];
      else {
        g_r[c] = (T)a.grad_in[2 * (3 * ind + c)];
        g_i[c] = (T)a.grad_in[2 * (3 * ind + c) + 1];
      }
    }
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  C *grid = (C *)a.grid;
  for (int l0 = 0; l0 < cut; l0++) {
    int g0 = (u[0] + l0) % n0;
    for (int l1 = 0; l1 < cut; l1++) {
      int g1 = (u[1] + l1) % n1;
      const T px = ws[l0], py = ws[cut + l1], dx = ws[3 * cut + l0], dy = ws[3 * cut + cut + l1];
      for (int l2 = 0; l2 < cut; l2++) {
        int g2 = (u[2] + l2) % n2;
        const T pz = ws[2 * cut + l2], dz = ws[3 * cut + 2 * cut + l2];
        C v;
        v.x = (T)0;
        v.y = (T)0;
        if (DF) {
          v.x += px * py * pz * f_r;
          v.y += px * py * pz * f_i;
        }
        if (DG) {
          T w0 = dx * py * pz, w1 = px * dy * pz, w2 = px * py * dz;
          v.x += w0 * g_r[0] + w1 * g_r[1] + w2 * g_r[2];
          v.y += w0 * g_i[0] + w1 * g_i[1] + w2 * g_i[2];
        }
        v.x *= scale;
        v.y *= scale;
        atomic_add_grid(&grid[((size_t)g0 * n1 + g1) * n2 + g2], v);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// dispatch
// ---------------------------------------------------------------------------
static const int kThreads = 256;

void choose_tiles(int cut, bool fp32, const int *n, int *T) {
  // largest cubic tile whose halo-padded region fits the shared-memory budget
  const size_t budget = fp32 ? 112 * 1024 : 136 * 1024;
  const size_t elem = fp32 ? 8 : 16;
  int t = 16;
  while (t > 1) {
    size_t r = (size_t)(t + cut - 1);
    if (r * r * r * elem <= budget) break;
    t >>= 1;
  }
  if (fp32 && t > 8) t = 8;
  for (int d = 0; d < 3; d++) {
    int td = t;
    while (td > 1 && td > n[d]) td >>= 1;
    T[d] = td;
  }
}

size_t conv_smem_bytes(const int *T, int cut, bool fp32, bool spread) {
  size_t vol = (size_t)(T[0] + cut - 1) * (T[1] + cut - 1) * (T[2] + cut - 1);
  size_t elem = fp32 ? 4 : 8;
  size_t region = vol * 2 * elem;
  size_t scratch = (size_t)(kThreads / 32) * (spread ? 6 : 9) * cut * elem;
  return region + scratch;
}

template <typename T, int CUT, int MODE>
static void run_interp_tile(const ConvArgs &a, cudaStream_t s) {
  size_t sm = conv_smem_bytes(a.bin.T, CUT, sizeof(T) == 4, false);
  static bool attr_done = false;
  if (!attr_done) {
    cudaFuncSetAttribute(k_interp_tile<T, CUT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr_done = true;
  }
  k_interp_tile<T, CUT, MODE><<<a.bin.max_subs, kThreads, sm, s>>>(a);
}

template <typename T, int CUT, int MODE>
static void run_spread_tile(const ConvArgs &a, cudaStream_t s) {
  size_t sm = conv_smem_bytes(a.bin.T, CUT, sizeof(T) == 4, true);
  static bool attr_done = false;
  if (!attr_done) {
    cudaFuncSetAttribute(k_spread_tile<T, CUT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr_done = true;
  }
  k_spread_tile<T, CUT, MODE><<<a.bin.max_subs, kThreads, sm, s>>>(a);
}

template <typename T, int MODE>
static bool interp_by_cut(const ConvArgs &a, cudaStream_t s) {
  switch (a.w.cut) {
    case 5: run_interp_tile<T, 5, MODE>(a, s); return true;
    case 7: run_interp_tile<T, 7, MODE>(a, s); return true;
    case 9: run_interp_tile<T, 9, MODE>(a, s); return true;
    case 11: run_interp_tile<T, 11, MODE>(a, s); return true;
    case 13: run_interp_tile<T, 13, MODE>(a, s); return true;
    case 15: run_interp_tile<T, 15, MODE>(a, s); return true;
    default: return false;
  }
}

template <typename T, int MODE>
static bool spread_by_cut(const ConvArgs &a, cudaStream_t s) {
  switch (a.w.cut) {
    case 5: run_spread_tile<T, 5, MODE>(a, s); return true;
    case 7: run_spread_tile<T, 7, MODE>(a, s); return true;
    case 9: run_spread_tile<T, 9, MODE>(a, s); return true;
    case 11: run_spread_tile<T, 11, MODE>(a, s); return true;
    case 13: run_spread_tile<T, 13, MODE>(a, s); return true;
    case 15: run_spread_tile<T, 15, MODE>(a, s); return true;
    default: return false;
  }
}

static bool tiles_usable(const ConvArgs &a) {
  size_t sm = conv_smem_bytes(a.bin.T, a.w.cut, false, false);
  return a.w.cut <= 15 && sm <= 200 * 1024;
}

template <typename T>
static void interp_t(const ConvArgs &a, int mode, cudaStream_t s) {
  if (a.M == 0) return;
  bool done = false;
  if (tiles_usable(a) || sizeof(T) == 4) {
    switch (mode) {
      case 1: done = interp_by_cut<T, 1>(a, s); break;
      case 2: done = interp_by_cut<T, 2>(a, s); break;
      case 3: done = interp_by_cut<T, 3>(a, s); break;
      case 4: done = interp_by_cut<T, 4>(a, s); break;
      default: break;
    }
  }
  if (done) return;
  unsigned bl = (unsigned)((a.M + 127) / 128);
  switch (mode) {
    case 1: k_interp_generic<T, 1><<<bl, 128, 0, s>>>(a); break;
    case 2: k_interp_generic<T, 2><<<bl, 128, 0, s>>>(a); break;
    case 3: k_interp_generic<T, 3><<<bl, 128, 0, s>>>(a); break;
    case 4: k_interp_generic<T, 4><<<bl, 128, 0, s>>>(a); break;
    default: break;
  }
}

template <typename T>
static void spread_t(const ConvArgs &a, int mode, cudaStream_t s) {
  if (a.M == 0) return;
  bool done = false;
  if (tiles_usable(a) || sizeof(T) == 4) {
    switch (mode) {
      case 1: done = spread_by_cut<T, 1>(a, s); break;
      case 2: done = spread_by_cut<T, 2>(a, s); break;
      case 3: done = spread_by_cut<T, 3>(a, s); break;
      default: break;
    }
  }
  if (done) return;
  unsigned bl = (unsigned)((a.M + 127) / 128);
  switch (mode) {
    case 1: k_spread_generic<T, 1><<<bl, 128, 0, s>>>(a); break;
    case 2: k_spread_generic<T, 2><<<bl, 128, 0, s>>>(a); break;
    case 3: k_spread_generic<T, 3><<<bl, 128, 0, s>>>(a); break;
    default: break;
  }
}

void launch_interp(const ConvArgs &a, int mode, bool fp32, cudaStream_t s) {
  if (fp32) interp_t<float>(a, mode, s);
  else interp_t<double>(a, mode, s);
}

void launch_spread(const ConvArgs &a, int mode, bool fp32, cudaStream_t s) {
  if (fp32) spread_t<float>(a, mode, s);
  else spread_t<double>(a, mode, s);
}

}  // namespace pg
