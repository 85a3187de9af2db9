// conv.cu -- the convolution with the window: the binning of nodes onto
// grid tiles, and the dispatch of interpolation B (grid -> nodes,
// pnfft_trafo) and spreading B^T (nodes -> grid, pnfft_adj) to the kernels:
//   * interp_line.cu: FP32-mixed B (f only) over lines of tiles with
//     register-resident grid columns (the transpose of the spreading);
//   * interp_line_g.cu: the same with the gradient (FP32-mixed);
//   * interp_group.cu: FP32-mixed B (f only), groups of nodes per warp;
//   * interp_tile.cuh (interp_tile_f32.cu, interp_tile_f64.cu): B, one warp
//     per node over a shared-memory copy of the tile's region;
//   * spread_line_f.cu: FP32-mixed B^T of f alone over lines of tiles with a
//     rotating register window of grid columns;
//   * spread_line.cuh (spread_line_f32.cu, spread_line_f64.cu): B^T over
//     lines of tiles with register-resident grid columns (FP64, gradients);
//   * generic.cu: one thread per node, any cutoff and grid.
//
// Reference: loop_over_particles_trafo / _adj (kernel/ndft-parallel.c:2703-3009)
// with the stencil loops of kernel/assign.c:478-1159.  The reference walks the
// nodes one by one over a ghost-celled local grid; here nodes are binned by
// the tile that holds their lowest stencil point (floor(n x) - m, wrapped mod
// n) with a counting sort, and the periodic ghost-cell exchange/reduce of the
// reference (ndft-parallel.c:2558, 2679) becomes the modulo wrap of the tile
// loads and commits.
#include <cuda_runtime.h>
#include <stdio.h>

#include "pg_conv.cuh"
#include "pg_index.cuh"
#include "pg_kernels.h"
#include "pg_math.cuh"

namespace pg {

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
      // (fnx - m) mod n: one add or subtract for the usual nodes (|n x| < n),
      // the 64-bit remainder otherwise
      long long w = fnx - m;
      if (w >= -nn[d] && w < 2LL * nn[d]) {
        int wi = (int)w;
        wi += wi < 0 ? nn[d] : 0;
        wi -= wi >= nn[d] ? nn[d] : 0;
        u[d] = wi;
      } else {
        w %= nn[d];
        if (w < 0) w += nn[d];
        u[d] = (int)w;
      }
      dist[d] = (T)fr;
    } else {
      AxisPos p = axis_pos(x[3 * j + d], nn[d], m, il);
      u[d] = p.u;
      dist[d] = (T)p.dist;
    }
  }
  const int t0 = u[0] / b.T[0], t1 = u[1] / b.T[1], t2 = u[2] / b.T[2];
  const int tile = (t0 * b.ntile[1] + t1) * b.ntile[2] + t2;
  const int l0 = u[0] - t0 * b.T[0], l1 = u[1] - t1 * b.T[1], l2 = u[2] - t2 * b.T[2];
  const int z = b.line_mode == BIN_LINE ? u[2] : l2;
  const int opk = l0 | (l1 << 8) | (z << 16);
  // group mode: 8x8x8 tiles cut into 4x4x2 blocks of 2x2x4 corners
  const int key = b.line_mode == BIN_GROUP ? tile * kBlocksPerTile + ((l0 >> 1) * 4 + (l1 >> 1)) * 2 + (l2 >> 2)
                                           : tile;
  b.key[j] = key;
  store_rec(rec_unsorted, j, dist, opk, T(0));
  b.rank[j] = atomicAdd(&b.count[key], 1);  // position of the node within its key
}

// three-phase exclusive scan of the tile counts and sub-problem counts
constexpr int kScanBlock = 2048;

__global__ void __launch_bounds__(256) k_bin_scan_a(Binning b, int *bsum) {
  __shared__ int ra[256], rb[256];
  const int lo = blockIdx.x * kScanBlock;
  int sa = 0, sb = 0;
  for (int i = lo + threadIdx.x; i < min(b.nkeys, lo + kScanBlock); i += 256) {
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
  if (tid == 1023) *(b.line_mode == BIN_LINE ? b.ntsub : b.nsub) = sb[1023];
}

__global__ void __launch_bounds__(256) k_bin_scan_c(Binning b, const int *bsum) {
  __shared__ int ca[kScanBlock], cb[kScanBlock];
  __shared__ int wa[8], wb[8];
  const int lo = blockIdx.x * kScanBlock, tid = threadIdx.x;
  const int n = min(kScanBlock, b.nkeys - lo);
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
  const int r = b.rank[j];
  const int pos = b.start[b.key[j]] + r;
  b.perm[pos] = (int)j;
  // group mode: every kGroupMax-th node of a block starts a group
  const int flag = (b.line_mode == BIN_GROUP && r % kGroupMax == 0) ? kGroupBit : 0;
  if (sizeof(T) == 4) {
    float4 v = ((const float4 *)rec_unsorted)[j];
    v.w = __int_as_float(__float_as_int(v.w) | flag);
    ((float4 *)b.rec)[pos] = v;
  } else {
    double4 v = ((const double4 *)rec_unsorted)[j];
    v.w = __longlong_as_double(__double_as_longlong(v.w) | flag);
    ((double4 *)b.rec)[pos] = v;
  }
}

// runs of at most sub_max nodes of one key (tile), into the list (tile, first, cnt)
__global__ void k_bin_subs(Binning b, int *tile, int *first, int *cntv) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.nkeys) return;
  int ns = b.nsub_tile[t], off = b.sub_off[t], st = b.start[t], c = b.count[t];
  for (int i = 0; i < ns; i++) {
    tile[off + i] = t;
    first[off + i] = st + i * b.sub_max;
    cntv[off + i] = min(b.sub_max, c - i * b.sub_max);
  }
}

// line and group modes: sub-problems over units of `group` consecutive keys
// (a line of tiles along axis 2, or the corner blocks of one tile); thread per
// unit.  `ordered`: sub-problem L is the first run of unit L (empty when the
// unit has no nodes) and further runs follow the nunits slots, so that CTAs
// take tiles / lines in grid order (neighbours share their halos in L2)
__global__ void k_bin_group_subs(Binning b, int64_t M, int group, int nunits, int ordered) {
  const int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nunits) return;
  const int first = b.start[L * group];
  const int end = (L + 1 < nunits) ? b.start[(L + 1) * group] : (int)M;
  const int cnt = end - first;
  if (ordered) {
    const int ns = cnt > 0 ? (cnt + b.sub_max - 1) / b.sub_max : 1;
    b.sub_tile[L] = L;
    b.sub_first[L] = first;
    b.sub_cnt[L] = min(b.sub_max, max(cnt, 0));
    const int off = ns > 1 ? nunits + atomicAdd(b.nsub + 1, ns - 1) : 0;
    for (int i = 1; i < ns; i++) {
      b.sub_tile[off + i - 1] = L;
      b.sub_first[off + i - 1] = first + i * b.sub_max;
      b.sub_cnt[off + i - 1] = min(b.sub_max, cnt - i * b.sub_max);
    }
    if (L == 0 || ns > 1) atomicAdd(b.nsub, (L == 0 ? nunits : 0) + ns - 1);
    return;
  }
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
  cudaMemsetAsync(b.count, 0, sizeof(int) * b.nkeys, s);
  const int th = 256;
  const unsigned bl = (unsigned)((a.M + th - 1) / th);
  if (a.M > 0) {
    if (fp32)
      k_bin_keys<float><<<bl, th, 0, s>>>(a.x, a.M, a.w.n[0], a.w.n[1], a.w.n[2], a.w.m, a.il, b, b.rec_tmp);
    else
      k_bin_keys<double><<<bl, th, 0, s>>>(a.x, a.M, a.w.n[0], a.w.n[1], a.w.n[2], a.w.m, a.il, b, b.rec_tmp);
  }
  const int nblk = (b.nkeys + kScanBlock - 1) / kScanBlock;
  k_bin_scan_a<<<nblk, 256, 0, s>>>(b, b.bsum);
  k_bin_scan_b<<<1, 1024, 0, s>>>(b, b.bsum, nblk);
  k_bin_scan_c<<<nblk, 256, 0, s>>>(b, b.bsum);
  if (a.M > 0) {
    if (fp32) k_bin_scatter<float><<<bl, th, 0, s>>>(a.M, b, b.rec_tmp);
    else k_bin_scatter<double><<<bl, th, 0, s>>>(a.M, b, b.rec_tmp);
  }
  if (b.line_mode != BIN_TILE) {
    const bool line = b.line_mode == BIN_LINE;
    const int group = line ? b.ntile[2] : kBlocksPerTile;
    const int nunits = line ? b.ntile[0] * b.ntile[1] : b.ntiles;
    if (line) k_bin_subs<<<(b.nkeys + 255) / 256, 256, 0, s>>>(b, b.tsub_tile, b.tsub_first, b.tsub_cnt);
    cudaMemsetAsync(b.nsub, 0, 2 * sizeof(int), s);
    k_bin_group_subs<<<(nunits + 255) / 256, 256, 0, s>>>(b, a.M, group, nunits, 1);
  } else {
    k_bin_subs<<<(b.nkeys + 255) / 256, 256, 0, s>>>(b, b.sub_tile, b.sub_first, b.sub_cnt);
  }
}

// ---------------------------------------------------------------------------
// dispatch
// ---------------------------------------------------------------------------
void choose_tiles(int cut, bool fp32, bool spread, bool f_only, int method, const int *n, int64_t M, int *T,
                  int *line_mode) {
  // Lines of 4x4x4-cell tiles along axis 2 (the record packs u2 in 15 bits)
  // for every kernel where the cutoff allows: the line kernels of B^T and of
  // the FP32-mixed B of f, and the one-warp-per-node B over each 4x4x4 tile's
  // (3+cutoff)^3 region for the other interpolations -- one binning serves both
  // directions.  Conv methods 2 and 3 of the FP32-mixed B take 8x8x8 tiles
  // (one warp per node; groups of nodes per warp for f alone with method 3).
  *line_mode = BIN_TILE;
  const bool lines_fit = n[0] >= 4 && n[1] >= 4 && n[2] >= 4 && n[2] < 32768 && cut <= 15;
  const bool tiles8 = !spread && fp32 && (method == 2 || method == 3);
  if (lines_fit && !tiles8) {
    T[0] = T[1] = T[2] = 4;
    *line_mode = BIN_LINE;
    return;
  }
  for (int d = 0; d < 3; d++) T[d] = n[d] >= 8 ? 8 : n[d];
  // method 3: groups of the nodes of 2x2x4 corner blocks when there are enough
  // of them (on average half a node per block or more); a group's z extent,
  // cut + 3, must fit the 16 lanes of a half-warp
  const int64_t ntiles = (int64_t)((n[0] + 7) / 8) * ((n[1] + 7) / 8) * ((n[2] + 7) / 8);
  if (!spread && fp32 && method == 3 && cut <= 13 && T[0] == 8 && T[1] == 8 && T[2] == 8 &&
      ntiles * kBlocksPerTile < (1 << 30) && 2 * M >= ntiles * kBlocksPerTile)
    *line_mode = BIN_GROUP;
}

// interpolation: 8x8x8 tiles; spreading: lines of 4x4x4 tiles
static bool tiles_usable(const ConvArgs &a) {
  if (a.bin.line_mode == BIN_LINE) return a.w.cut <= 15 && a.bin.T[0] == 4 && a.bin.T[1] == 4 && a.bin.T[2] == 4;
  return a.w.cut <= 15 && a.bin.T[0] == 8 && a.bin.T[1] == 8 && a.bin.T[2] == 8;
}

bool interp_line_chosen(const ConvArgs &a, int mode, bool fp32) {
  const int c = a.w.cut;
  return a.M > 0 && fp32 && mode == 1 && a.method == 0 && a.bin.line_mode == BIN_LINE && tiles_usable(a) &&
         (c == 5 || c == 7 || c == 9 || c == 11 || c == 13);
}

bool spread_line_f_chosen(const ConvArgs &a, int mode, bool fp32) {
  const int c = a.w.cut;
  return a.M > 0 && fp32 && mode == 1 && a.method == 0 && a.bin.line_mode == BIN_LINE && tiles_usable(a) &&
         (c == 5 || c == 7 || c == 9 || c == 11 || c == 13);
}

__global__ void k_store_conv_args(ConvArgs a, ConvArgs *dst) {
  if (threadIdx.x == 0) *dst = a;
}

void store_conv_args(const ConvArgs &a, ConvArgs *dst, cudaStream_t s) { k_store_conv_args<<<1, 32, 0, s>>>(a, dst); }

int launch_interp(const ConvArgs &a, int mode, bool fp32, cudaStream_t s) {
  if (a.M == 0) return CONV_NONE;
  if (fp32 && mode == 1 && a.method == 0 && a.bin.line_mode == BIN_LINE && tiles_usable(a) &&
      launch_interp_line(a, s))
    return CONV_LINE;
  if (fp32 && (mode == 2 || mode == 3) && a.method == 0 && a.bin.line_mode == BIN_LINE && tiles_usable(a) &&
      a.w.cut <= 13 && launch_interp_line_g(a, mode, s))
    return CONV_LINE;
  if (!a.generic && a.bin.line_mode == BIN_LINE && tiles_usable(a)) {
    // one warp per node over the 4x4x4 tiles of the line binning
    ConvArgs t = a;
    t.bin.sub_tile = a.bin.tsub_tile;
    t.bin.sub_first = a.bin.tsub_first;
    t.bin.sub_cnt = a.bin.tsub_cnt;
    t.bin.nsub = a.bin.ntsub;
    t.bin.max_subs = a.bin.max_tsubs;
    if (fp32 ? launch_interp_tile_f32(t, mode, s) : launch_interp_tile_f64(t, mode, s)) return CONV_TILE;
  }
  if (fp32 && mode == 1 && !a.generic && a.bin.line_mode == BIN_GROUP && tiles_usable(a) &&
      a.bin.sub_max <= kGroupSubMax && launch_interp_group(a, s))
    return CONV_GROUP;
  if (!a.generic && a.bin.line_mode != BIN_LINE && tiles_usable(a) &&
      (fp32 ? launch_interp_tile_f32(a, mode, s) : launch_interp_tile_f64(a, mode, s)))
    return CONV_TILE;
  launch_interp_generic(a, mode, fp32, s);
  return CONV_GENERIC;
}

int launch_spread(const ConvArgs &a, int mode, bool fp32, cudaStream_t s) {
  if (a.M == 0) return CONV_NONE;
  if (fp32 && mode == 1 && a.method == 0 && a.bin.line_mode == BIN_LINE && tiles_usable(a) &&
      launch_spread_line_f(a, s))
    return CONV_LINE;
  if (!a.generic && a.bin.line_mode == BIN_LINE && tiles_usable(a) &&
      (fp32 ? launch_spread_line_f32(a, mode, s) : launch_spread_line_f64(a, mode, s)))
    return CONV_LINE;
  launch_spread_generic(a, mode, fp32, s);
  return CONV_GENERIC;
}

}  // namespace pg
