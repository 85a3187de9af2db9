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

#include <atomic>

#include "pg_index.cuh"
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
// ---------------------------------------------------------------------------
// binning
//
// k_bin_keys computes, once per node, the lowest stencil index u (bit-exact)
// and the fractional positions, writes the node record (unsorted) and counts
// nodes per tile (the count before its own increment is the node's rank in
// the tile); a three-phase scan gives tile starts and the sub-problem list;
// k_bin_scatter moves perm and records to start[tile] + rank.
// For the FP32-mixed form without interlacing, floor(fl(n x)) is evaluated
// with integer arithmetic on the bits of x (the FP64 pipe of GB300 is slow):
// the exact product n*M_x (<= 73 bits) is rounded to 53 bits with ties to
// even -- which is fl(n x) -- and split into integer and fractional parts.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void store_rec(void *rec, int64_t pos, const float *dist, int opk, float) {
  ((float4 *)rec)[pos] = make_float4(dist[0], dist[1], dist[2], __int_as_float(opk));
}
__device__ __forceinline__ void store_rec(void *rec, int64_t pos, const double *dist, int opk, double) {
  ((double4 *)rec)[pos] = make_double4(dist[0], dist[1], dist[2], __longlong_as_double((long long)opk));
}

template <typename T>
__global__ void k_bin_keys(const double *__restrict__ x, int64_t M, int n0, int n1, int n2, int m, int il,
                           Binning b, void *__restrict__ rec_unsorted) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const int nn[3] = {n0, n1, n2};
  T dist[3];
  int u[3];
  for (int d = 0; d < 3; d++) {
    if (sizeof(T) == 4 && !il) {
      long long fnx;
      float fr;
      nx_exact(x[3 * j + d], nn[d], &fnx, &fr);
      long long w = (fnx - m) % nn[d];
      if (w < 0) w += nn[d];
      u[d] = (int)w;
      dist[d] = (T)fr;
    } else {
      AxisPos p = axis_pos(x[3 * j + d], nn[d], m, il);
      u[d] = p.u;
      dist[d] = (T)p.dist;
    }
  }
  const int t0 = u[0] / b.T[0], t1 = u[1] / b.T[1], t2 = u[2] / b.T[2];
  const int tile = (t0 * b.ntile[1] + t1) * b.ntile[2] + t2;
  const int z = b.line_mode ? u[2] : u[2] - t2 * b.T[2];
  const int opk = (u[0] - t0 * b.T[0]) | ((u[1] - t1 * b.T[1]) << 8) | (z << 16);
  b.key[j] = tile;
  store_rec(rec_unsorted, j, dist, opk, T(0));
  b.rank[j] = atomicAdd(&b.count[tile], 1);  // position of the node within its tile
}

// three-phase exclusive scan of the tile counts and sub-problem counts
constexpr int kScanBlock = 2048;

__global__ void __launch_bounds__(256) k_bin_scan_a(Binning b, int *bsum) {
  __shared__ int ra[256], rb[256];
  const int lo = blockIdx.x * kScanBlock;
  int sa = 0, sb = 0;
  for (int i = lo + threadIdx.x; i < min(b.ntiles, lo + kScanBlock); i += 256) {
    int c = b.count[i];
    sa += c;
    sb += (c + b.sub_max - 1) / b.sub_max;
  }
  ra[threadIdx.x] = sa;
  rb[threadIdx.x] = sb;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      ra[threadIdx.x] += ra[threadIdx.x + o];
      rb[threadIdx.x] += rb[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    bsum[2 * blockIdx.x] = ra[0];
    bsum[2 * blockIdx.x + 1] = rb[0];
  }
}

__global__ void __launch_bounds__(1024) k_bin_scan_b(Binning b, int *bsum, int nblk) {
  __shared__ int sa[1024], sb[1024];
  const int tid = threadIdx.x;
  const int chunk = (nblk + 1023) / 1024;
  const int lo = min(nblk, tid * chunk), hi = min(nblk, lo + chunk);
  int a = 0, c = 0;
  for (int i = lo; i < hi; i++) {
    a += bsum[2 * i];
    c += bsum[2 * i + 1];
  }
  sa[tid] = a;
  sb[tid] = c;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    int va = (tid >= off) ? sa[tid - off] : 0, vb = (tid >= off) ? sb[tid - off] : 0;
    __syncthreads();
    sa[tid] += va;
    sb[tid] += vb;
    __syncthreads();
  }
  int pa = sa[tid] - a, pb = sb[tid] - c;
  for (int i = lo; i < hi; i++) {
    int x0 = bsum[2 * i], x1 = bsum[2 * i + 1];
    bsum[2 * i] = pa;
    bsum[2 * i + 1] = pb;
    pa += x0;
    pb += x1;
  }
  if (tid == 1023) *b.nsub = sb[1023];
}

__global__ void __launch_bounds__(256) k_bin_scan_c(Binning b, const int *bsum) {
  __shared__ int ca[kScanBlock], cb[kScanBlock];
  __shared__ int wa[8], wb[8];
  const int lo = blockIdx.x * kScanBlock, tid = threadIdx.x;
  const int n = min(kScanBlock, b.ntiles - lo);
  for (int i = tid; i < kScanBlock; i += 256) {
    int c = (i < n) ? b.count[lo + i] : 0;
    ca[i] = c;
    cb[i] = (c + b.sub_max - 1) / b.sub_max;
  }
  __syncthreads();
  // each thread scans 8 consecutive entries, then a warp-level scan of the thread sums
  const int k0 = tid * 8;
  int ta = 0, tb = 0;
  for (int k = 0; k < 8; k++) {
    ta += ca[k0 + k];
    tb += cb[k0 + k];
  }
  const int lane = tid & 31, w = tid >> 5;
  int xa = ta, xb = tb;
  for (int o = 1; o < 32; o <<= 1) {
    int ya = __shfl_up_sync(0xffffffffu, xa, o), yb = __shfl_up_sync(0xffffffffu, xb, o);
    if (lane >= o) {
      xa += ya;
      xb += yb;
    }
  }
  if (lane == 31) {
    wa[w] = xa;
    wb[w] = xb;
  }
  __syncthreads();
  int oa = bsum[2 * blockIdx.x], ob = bsum[2 * blockIdx.x + 1];
  for (int v = 0; v < w; v++) {
    oa += wa[v];
    ob += wb[v];
  }
  oa += xa - ta;
  ob += xb - tb;
  for (int k = 0; k < 8; k++) {
    const int i = k0 + k;
    if (i < n) {
      b.start[lo + i] = oa;
      b.nsub_tile[lo + i] = cb[i];
      b.sub_off[lo + i] = ob;
    }
    oa += ca[i];
    ob += cb[i];
  }
}

template <typename T>
__global__ void k_bin_scatter(int64_t M, Binning b, const void *__restrict__ rec_unsorted) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const int pos = b.start[b.key[j]] + b.rank[j];
  b.perm[pos] = (int)j;
  if (sizeof(T) == 4) ((float4 *)b.rec)[pos] = ((const float4 *)rec_unsorted)[j];
  else ((double4 *)b.rec)[pos] = ((const double4 *)rec_unsorted)[j];
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

// line mode: one sub-problem list over lines of tiles along axis 2 (thread per line)
__global__ void k_bin_line_subs(Binning b, int64_t M) {
  const int nlines = b.ntile[0] * b.ntile[1];
  const int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nlines) return;
  const int first = b.start[L * b.ntile[2]];
  const int end = (L + 1 < nlines) ? b.start[(L + 1) * b.ntile[2]] : (int)M;
  const int cnt = end - first;
  if (cnt <= 0) return;
  const int ns = (cnt + b.sub_max - 1) / b.sub_max;
  const int off = atomicAdd(b.nsub, ns);
  for (int i = 0; i < ns; i++) {
    b.sub_tile[off + i] = L;
    b.sub_first[off + i] = first + i * b.sub_max;
    b.sub_cnt[off + i] = min(b.sub_max, cnt - i * b.sub_max);
  }
}

void bin_nodes(const ConvArgs &a, bool fp32, cudaStream_t s) {
  const Binning &b = a.bin;
  cudaMemsetAsync(b.count, 0, sizeof(int) * b.ntiles, s);
  const int th = 256;
  const unsigned bl = (unsigned)((a.M + th - 1) / th);
  if (a.M > 0) {
    if (fp32)
      k_bin_keys<float><<<bl, th, 0, s>>>(a.x, a.M, a.w.n[0], a.w.n[1], a.w.n[2], a.w.m, a.il, b, b.rec_tmp);
    else
      k_bin_keys<double><<<bl, th, 0, s>>>(a.x, a.M, a.w.n[0], a.w.n[1], a.w.n[2], a.w.m, a.il, b, b.rec_tmp);
  }
  const int nblk = (b.ntiles + kScanBlock - 1) / kScanBlock;
  k_bin_scan_a<<<nblk, 256, 0, s>>>(b, b.bsum);
  k_bin_scan_b<<<1, 1024, 0, s>>>(b, b.bsum, nblk);
  k_bin_scan_c<<<nblk, 256, 0, s>>>(b, b.bsum);
  if (a.M > 0) {
    if (fp32) k_bin_scatter<float><<<bl, th, 0, s>>>(a.M, b, b.rec_tmp);
    else k_bin_scatter<double><<<bl, th, 0, s>>>(a.M, b, b.rec_tmp);
  }
  if (b.line_mode) {
    const int nlines = b.ntile[0] * b.ntile[1];
    cudaMemsetAsync(b.nsub, 0, sizeof(int), s);
    k_bin_line_subs<<<(nlines + 255) / 256, 256, 0, s>>>(b, a.M);
  } else {
    k_bin_subs<<<(b.ntiles + 255) / 256, 256, 0, s>>>(b);
  }
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
// shared helpers of the tiled kernels (8x8x8-cell tiles, compile-time cutoff)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void window_formula(const WindowArgs &w, int t, int s, float dist, int nder, float *out) {
  window_eval_f(w.kind, w.m, w.wf[t], w.m - s, dist, nder, out);
}
__device__ __forceinline__ void window_formula(const WindowArgs &w, int t, int s, double dist, int nder,
                                               double *out) {
  window_eval<double>(w.kind, w.m, (double)w.n[t], w.b[t], dist + (double)(w.m - s), (double)s - dist, nder, out);
}

// FP32: Horner on the fitted polynomial of stencil point s (16 FMAs per value)
__device__ __forceinline__ float poly_eval(const float *row, float u) {
  const float4 *r = (const float4 *)row;
  const float4 c0 = __ldg(r), c1 = __ldg(r + 1), c2 = __ldg(r + 2), c3 = __ldg(r + 3);
  float h = c3.w;
  h = fmaf(h, u, c3.z);
  h = fmaf(h, u, c3.y);
  h = fmaf(h, u, c3.x);
  h = fmaf(h, u, c2.w);
  h = fmaf(h, u, c2.z);
  h = fmaf(h, u, c2.y);
  h = fmaf(h, u, c2.x);
  h = fmaf(h, u, c1.w);
  h = fmaf(h, u, c1.z);
  h = fmaf(h, u, c1.y);
  h = fmaf(h, u, c1.x);
  h = fmaf(h, u, c0.w);
  h = fmaf(h, u, c0.z);
  h = fmaf(h, u, c0.y);
  return fmaf(h, u, c0.x);
}

// psi (and derivatives up to nder) of stencil point s on axis t for a node at
// fractional position dist, from the interpolation table, the fitted
// polynomial (FP32) or the formula
template <typename T>
__device__ __forceinline__ void window_point(const WindowArgs &w, int t, int s, T dist, int nder, T *out) {
  if constexpr (sizeof(T) == 4) {
    // the Bessel-I0 window jumps from 1/2 to 0 at y = m (s = 0, dist = 0)
    if (w.poly && w.intpol_order < 0 && !(w.kind == WIN_BESSEL_I0 && s == 0 && dist == 0.f)) {
      const float u = dist - 0.5f;
      for (int d = 0; d <= nder; d++) out[d] = poly_eval(w.poly + ((d * 3 + t) * w.cut + s) * kPolyCoef, u);
      return;
    }
  }
  if (w.intpol_order >= 0) {
    T dK = dist * (T)w.intpol_K;
    int k = (int)floor(dK);
    T dk = dK - (T)k;
    size_t base = ((size_t)k * w.cut + s) * (size_t)(w.intpol_order + 1);
    for (int d = 0; d <= nder; d++) out[d] = intpol<T>(w.intpol_order, (const T *)w.tab[d][t] + base, dk);
  } else {
    window_formula(w, t, s, dist, nder, out);
  }
}

__device__ __forceinline__ void unpack_corner(int pk, int *o) {
  o[0] = pk & 0xff;
  o[1] = (pk >> 8) & 0xff;
  o[2] = (pk >> 16) & 0xff;
}

__device__ __forceinline__ void load_rec_raw(const void *rec, int pos, float *d, int *pk) {
  float4 r = ((const float4 *)rec)[pos];
  d[0] = r.x;
  d[1] = r.y;
  d[2] = r.z;
  *pk = __float_as_int(r.w);
}
__device__ __forceinline__ void load_rec_raw(const void *rec, int pos, double *d, int *pk) {
  double4 r = ((const double4 *)rec)[pos];
  d[0] = r.x;
  d[1] = r.y;
  d[2] = r.z;
  *pk = (int)__double_as_longlong(r.w);
}

// ---------------------------------------------------------------------------
// interpolation B, tiled.  The CTA stages its tile's (8+2m)^3 region in
// shared memory, then walks its nodes in batches: (1) all threads evaluate
// the window values of the batch (3 x cutoff per node and derivative), (2)
// one warp per node sums the 13^3 stencil -- lanes (row = lane/16, col =
// lane%16) read two z-rows of 13 consecutive grid values per step, with the
// x-window in registers -- and reduces with shuffles, (3) the batch's results
// are converted and written by all threads.
// ---------------------------------------------------------------------------
template <typename T, int CUT, int MODE>
struct InterpGeom {
  static constexpr bool DF = (MODE & 1) != 0, DG = (MODE & 2) != 0, DH = (MODE & 4) != 0;
  static constexpr int NDER = DH ? 2 : (DG ? 1 : 0);
  static constexpr int R = 8 + CUT - 1, PL = R * R, VOL = R * R * R;
  static constexpr int NV = 3 * CUT * (NDER + 1);
  static constexpr int NC = (DF ? 1 : 0) + (DG ? 3 : 0) + (DH ? 6 : 0);
  static constexpr int NBI = sizeof(T) == 4 ? 48 : 32;
  static constexpr size_t SMEM = (size_t)VOL * 2 * sizeof(T) + (size_t)NBI * (NV + 2 * NC + 4) * sizeof(T) +
                                 (size_t)NBI * 2 * sizeof(int);
};

template <typename T, int CUT, int MODE>
__global__ void __launch_bounds__(256) k_interp_tile(ConvArgs a) {
  typedef typename Cplx<T>::type C;
  typedef InterpGeom<T, CUT, MODE> G;
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
  int base[3];
  tile_base(b, tile, base);
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  const int tid = threadIdx.x;
  const C *grid = (const C *)a.grid;
  for (int i = tid; i < VOL; i += blockDim.x) {
    int c = i % R, q = i / R;
    int bb = q % R, aa = q / R;
    int g0 = base[0] + aa, g1 = base[1] + bb, g2 = base[2] + c;
    if (g0 >= n0) g0 %= n0;
    if (g1 >= n1) g1 %= n1;
    if (g2 >= n2) g2 %= n2;
    C v = grid[((size_t)g0 * n1 + g1) * n2 + g2];
    if (a.real_only) v.y = (T)0;
    reg[i] = v;
  }
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
      T px[CUT], dpx[CUT], ddpx[CUT];
#pragma unroll
      for (int l = 0; l < CUT; l++) {
        px[l] = wv[l];
        if (NDER >= 1) dpx[l] = wv[3 * CUT + l];
        if (NDER >= 2) ddpx[l] = wv[6 * CUT + l];
      }
      T af_r = 0, af_i = 0;
      T ag_r[3] = {0, 0, 0}, ag_i[3] = {0, 0, 0};
      T ah_r[6] = {0, 0, 0, 0, 0, 0}, ah_i[6] = {0, 0, 0, 0, 0, 0};
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
            T s_r = 0, s_i = 0, sd_r = 0, sd_i = 0, sdd_r = 0, sdd_i = 0;
#pragma unroll
            for (int l0 = 0; l0 < CUT; l0++) {
              const C g = p[l0 * PL];
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
      }
      T *res = s_res + i * 2 * NC;
      int c = 0;
      if (DF) {
        T r = warp_sum(af_r), im = warp_sum(af_i);
        if (lane == 0) {
          res[0] = r * scale;
          res[1] = im * scale;
        }
        c = 1;
      }
      if (DG) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          T r = warp_sum(ag_r[k]), im = warp_sum(ag_i[k]);
          if (lane == 0) {
            res[2 * (c + k)] = r * scale;
            res[2 * (c + k) + 1] = im * scale;
          }
        }
      }
      if (DH) {
#pragma unroll
        for (int k = 0; k < 6; k++) {
          T r = warp_sum(ah_r[k]), im = warp_sum(ah_i[k]);
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
  for (int e = 0; e < 3 * cut; e++) {
    int t = e / cut, s = e - t * cut;
    T out[3] = {(T)0, (T)0, (T)0};
    window_point<T>(a.w, t, s, (T)dist[t], NDER, out);
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
    window_point<T>(a.w, t, s, (T)dist[t], NDER, out);
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

// adds (r0 + i i0) at z and (r1 + i i1) at z+1 of one grid column (z even)
__device__ __forceinline__ void commit_pair(float2 *col, int z, int n2, bool vec, float r0, float i0, float r1,
                                            float i1) {
  if (r0 == 0.f && i0 == 0.f && r1 == 0.f && i1 == 0.f) return;
  if (vec) {
    atomicAdd((float4 *)(col + z % n2), make_float4(r0, i0, r1, i1));
  } else {
    if (r0 != 0.f || i0 != 0.f) atomicAdd(col + z % n2, make_float2(r0, i0));
    if (r1 != 0.f || i1 != 0.f) atomicAdd(col + (z + 1) % n2, make_float2(r1, i1));
  }
}
__device__ __forceinline__ void commit_pair(double2 *col, int z, int n2, bool, double r0, double i0, double r1,
                                            double i1) {
  if (r0 != 0.0 || i0 != 0.0) atomic_add_grid(col + z % n2, make_double2(r0, i0));
  if (r1 != 0.0 || i1 != 0.0) atomic_add_grid(col + (z + 1) % n2, make_double2(r1, i1));
}

template <typename T, int CUT, int MODE>
__global__ void __launch_bounds__(LineGeom<CUT>::THREADS, sizeof(T) == 4 ? 5 : 1) k_spread_line(ConvArgs a) {
  typedef typename Cplx<T>::type C;
  typedef LineGeom<CUT> G;
  constexpr int TL = G::TL, R = G::R, HR = G::HR, W = G::W, WP = G::WP, CP = G::CP, WREC = G::WREC;
  constexpr bool DF = (MODE & 1) != 0, DG = (MODE & 2) != 0;
  constexpr int NDER = DG ? 1 : 0;
  constexpr int NB = sizeof(T) == 4 ? 64 : 32;  // nodes per batch
  constexpr int WSZ0 = (DG ? 2 : 1) * WREC;
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
  const int t1 = line % b.ntile[1], t0 = line / b.ntile[1];
  const int tid = threadIdx.x, nth = blockDim.x;
  const bool active = tid < R * HR;
  const int ca = active ? tid / HR : 0, cb = active ? tid % HR : 0;
  const int n0 = a.w.n[0], n1 = a.w.n[1], n2 = a.w.n[2];
  const size_t gx = (size_t)((t0 * TL + ca) % n0) * n1;
  C *col[2] = {(C *)a.grid + (gx + (t1 * TL + cb) % n1) * n2, (C *)a.grid + (gx + (t1 * TL + cb + HR) % n1) * n2};
  const bool vec = (n2 & 1) == 0;
  T acc_r[2][W], acc_i[2][W];
#pragma unroll
  for (int c = 0; c < 2; c++)
#pragma unroll
    for (int z = 0; z < W; z++) acc_r[c][z] = acc_i[c][z] = (T)0;
  int zslab = -1, since = 0;
  const T scale = a.use_il ? (T)0.5 : (T)1;
  // commit values [z0, z1) of both columns at grid z = zb + z
  auto commit = [&](int zb, int z0, int z1) {
#pragma unroll
    for (int c = 0; c < 2; c++)
#pragma unroll
      for (int z = 0; z < W; z += 2)
        if (z >= z0 && z < z1)
          commit_pair(col[c], zb + z, n2, vec, acc_r[c][z], acc_i[c][z], acc_r[c][z + 1], acc_i[c][z + 1]);
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
    for (int v = tid; v < nb * WP; v += nth) {
      const int i = v / WP, z = v - i * WP;
      s_w[i][z] = (T)0;
      if (DG) s_w[i][WREC + z] = (T)0;
    }
    __syncthreads();
    // --- window values: all threads over (node, axis, stencil point) ------------
    // node-fastest (broadcast polynomial rows); the odd row stride in 16-byte
    // units keeps these stores to at most 4-way bank conflicts
#pragma unroll 2  // two independent polynomial chains per thread
    for (int v = tid; v < NB * 3 * CUT; v += nth) {
      const int e = v / NB, i = v - e * NB;
      if (i >= nb) continue;
      const int t = e / CUT, sidx = e - t * CUT;
      T out[3];
      window_point<T>(a.w, t, sidx, s_d[i][t], NDER, out);
      const int pos = (t == 2) ? ((s_o[i] >> 16) & (TL - 1)) + sidx : WP + t * CP + sidx;
      s_w[i][pos] = out[0];
      if (DG) s_w[i][WREC + pos] = out[1];
    }
    __syncthreads();
    // --- accumulate, sliding the z window ----------------------------------------
    if (since >= kFlushNodes) {
      commit(zslab * TL, 0, W);
#pragma unroll
      for (int c = 0; c < 2; c++)
#pragma unroll
        for (int z = 0; z < W; z++) acc_r[c][z] = acc_i[c][z] = (T)0;
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
              for (int z = 0; z < W; z++) acc_r[c][z] = acc_i[c][z] = (T)0;
          } else {
            for (int q = 0; q < steps; q++) {
              commit((zslab + q) * TL, 0, TL);
#pragma unroll
              for (int c = 0; c < 2; c++) {
#pragma unroll
                for (int z = 0; z < W - TL; z++) {
                  acc_r[c][z] = acc_r[c][z + TL];
                  acc_i[c][z] = acc_i[c][z + TL];
                }
#pragma unroll
                for (int z = W - TL; z < W; z++) acc_r[c][z] = acc_i[c][z] = (T)0;
              }
            }
          }
        }
        zslab = slab;
        since = 0;
      }
      since++;
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
            for (int z = 0; z < W; z++) {
              acc_r[c][z] += h1r * pz[z];
              acc_i[c][z] += h1i * pz[z];
            }
            if (DG) {
              const T h2r = g2r * py, h2i = g2i * py;
#pragma unroll
              for (int z = 0; z < W; z++) {
                acc_r[c][z] += h2r * dz[z];
                acc_i[c][z] += h2i * dz[z];
              }
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

// ---------------------------------------------------------------------------
// dispatch
// ---------------------------------------------------------------------------
static const int kThreads = 256;

void choose_tiles(int cut, bool fp32, bool spread, const int *n, int *T, int *line_mode) {
  // interpolation: 8x8x8 cells per tile, the CTA stages the (8+2m)^3 region
  // in shared memory (FP64, m=7: 170 KB).  Spreading: lines of 4x4x4-cell
  // tiles along axis 2 (k_spread_line); the record packs u2 in 15 bits.
  (void)fp32;
  *line_mode = 0;
  if (spread && cut <= 15 && n[0] >= 4 && n[1] >= 4 && n[2] >= 4 && n[2] < 32768) {
    T[0] = T[1] = T[2] = 4;
    *line_mode = 1;
    return;
  }
  for (int d = 0; d < 3; d++) T[d] = n[d] >= 8 ? 8 : n[d];
}

template <typename T, int CUT, int MODE>
static void run_interp_tile(const ConvArgs &a, cudaStream_t s) {
  const size_t sm = InterpGeom<T, CUT, MODE>::SMEM;
  // the shared-memory opt-in is a per-device attribute of the kernel
  static std::atomic<unsigned long long> attr_done{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(attr_done.load() & bit)) {
    cudaFuncSetAttribute(k_interp_tile<T, CUT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr_done.fetch_or(bit);
  }
  k_interp_tile<T, CUT, MODE><<<a.bin.max_subs, kThreads, sm, s>>>(a);
}

template <typename T, int CUT, int MODE>
static void run_spread_tile(const ConvArgs &a, cudaStream_t s) {
  k_spread_line<T, CUT, MODE><<<a.bin.max_subs, LineGeom<CUT>::THREADS, 0, s>>>(a);
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

// interpolation: 8x8x8 tiles; spreading: lines of 4x4x4 tiles
static bool tiles_usable(const ConvArgs &a) {
  if (a.bin.line_mode) return a.w.cut <= 15 && a.bin.T[0] == 4 && a.bin.T[1] == 4 && a.bin.T[2] == 4;
  return a.w.cut <= 15 && a.bin.T[0] == 8 && a.bin.T[1] == 8 && a.bin.T[2] == 8;
}

template <typename T>
static void interp_t(const ConvArgs &a, int mode, cudaStream_t s) {
  if (a.M == 0) return;
  bool done = false;
  if (!a.generic && !a.bin.line_mode && tiles_usable(a)) {
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
  if (!a.generic && a.bin.line_mode && tiles_usable(a)) {
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
