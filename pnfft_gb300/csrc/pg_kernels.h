// pg_kernels.h -- argument blocks and launchers of the device kernels.
// Included by the .cu files and by the host engine; no CUDA types appear in
// the launcher signatures except cudaStream_t.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pg_math.cuh"

namespace pg {

// Window description shared by the convolution kernels.
struct WindowArgs {
  int kind;           // pg::WindowKind
  int m, cut;         // cutoff = 2m+1
  int n[3];           // oversampled grid
  double b[3];        // shape parameters
  WinF wf[3];         // FP32 constants of each axis for the FP32-mixed kernels
  int intpol_order;   // -1: evaluate directly; 0..3: tabulated (PNFFT_PRE_*_PSI)
  int intpol_K;       // samples per grid cell of the tables
  const void *tab[3][3];  // [derivative][axis], element type = compute precision
  // FP32-mixed without PRE_*_PSI tables: per stencil point s a polynomial
  // in u = dist - 1/2 for psi and its two derivatives, fitted on the host in
  // FP64 (times 2^-kscale); layout [der][axis][s][16], poly_ncoef (12 or 16)
  // coefficients used, the rest zero
  const float *poly;
  int poly_ncoef;
  // the same polynomials in pairs of stencil points (points 2cp and 2cp + 1,
  // zero beyond the cutoff): row r = 3 der + axis, coefficient k of both at
  // poly_pp[((r * NP + cp) * 16 + k) * 2 + {0, 1}], NP = (cut + 1) / 2
  const float *poly_pp;
};
constexpr int kPolyCoef = 16;

// Node binning onto grid tiles (one tile = T0 x T1 x T2 cells of lowest
// stencil index).  A sub-problem is a run of at most `sub_max` nodes of one
// tile; one CTA handles one sub-problem.  In line mode a sub-problem is a run
// of the nodes of one line of tiles along axis 2 (the tiles with the same
// t0, t1, which the sort keeps consecutive and in slab order), and the
// records carry the full lowest z index u2 instead of the in-tile offset; a
// second list cuts the same sorted nodes by tile, so that every kernel can run
// on a line binning and one binning serves both directions.
// In group mode (FP32-mixed interpolation, conv method 3) the sort key is finer: the tile
// and the 2x2x4 block of stencil corners within it (32 keys per tile), and
// the record of every kGroupMax-th node of a block (by rank) carries a
// group-start bit, so that the nodes of one block are consecutive and cut
// into groups of at most kGroupMax nodes whose stencils overlap.
enum BinMode { BIN_TILE = 0, BIN_LINE = 1, BIN_GROUP = 2 };
constexpr int kBlocksPerTile = 32;  // 2x2x4 corner blocks of an 8x8x8 tile
constexpr int kGroupMax = 4;        // nodes of one block interpolated together
constexpr int kGroupBit = 1 << 24;  // record flag: first node of a group
constexpr int kGroupSubMax = 1024;  // nodes per sub-problem of the grouped interpolation

struct Binning {
  int T[3], ntile[3];
  int ntiles, sub_max, max_subs;
  int max_tsubs;   // line mode: capacity of the tile sub-problem list below
  int line_mode;   // BinMode
  int nkeys;       // sort keys: ntiles, or ntiles * kBlocksPerTile in group mode
  int *key;        // [M] sort key of each node
  int *perm;       // [M] nodes sorted by key
  int *count;      // [nkeys]
  int *start;      // [nkeys]
  int *rank;       // [M] position of each node within its key
  int *nsub_tile;  // [nkeys]
  int *sub_off;    // [nkeys]
  int *sub_tile;   // [max_subs]
  int *sub_first;  // [max_subs]
  int *sub_cnt;    // [max_subs]
  int *nsub;       // [2] sub-problem count; [1]: runs beyond the first per unit (group mode)
  // line mode: the same sorted nodes cut into runs of one 4x4x4 tile (at most
  // sub_max nodes each), for the one-warp-per-node interpolation kernels
  int *tsub_tile, *tsub_first, *tsub_cnt;  // [max_tsubs]
  int *ntsub;                              // [1]
  void *rec;       // [M] node records in tile order: float4 (FP32-mixed) or double4
                   // {dist0, dist1, dist2, local stencil corner o0 | o1<<8 | o2<<16}
  void *rec_tmp;   // [M] the same records in node order (before the scatter)
  int *bsum;       // [2 * ceil(nkeys / 2048)] scan block sums
};

// One convolution (B or B^T) launch.
struct ConvArgs {
  WindowArgs w;
  int use_il, il;   // interlacing: 0.5 scale / shifted pass
  int real_only;    // read only the real parts of the grid (c2r and the
                    // c2c + PNFFT_PRE_QUAD_PSI behaviour of the reference)
  int real_io;      // node arrays are real (c2r) instead of complex
  int accum;        // add into the node outputs (else store): ACCUMULATED, 2nd interlaced pass
  int generic;      // use the one-thread-per-node kernels (set per plan, e.g. by an autotuner)
  int method;       // the plan's conv method (pnfft_gb300_set_conv_method)
  int64_t M;
  const double *x;  // [M][3]
  void *grid;       // n0*n1*n2 complex in compute precision, natural order
  // node arrays (double, complex interleaved unless real_io), element ind = j*stride + offset
  const double *f_in, *grad_in;
  double *f_out, *grad_out, *hess_out;
  int64_t offset, stride;
  Binning bin;
};

// One launch over the line sub-problems of several calls (batched
// convolutions, engine.cu): block k runs sub-problem k - first[i] of item i,
// first[i] <= k < first[i + 1]; each item's ConvArgs sits in device memory
// (written on the stream by store_conv_args) so that a captured graph replays
// the same arguments.
constexpr int kMultiItems = 64;
struct MultiConv {
  const ConvArgs *args[kMultiItems];
  int first[kMultiItems + 1];
  int n;
};

// Launchers (conv.cu).  `fp32` selects the FP32-mixed kernels.  `mode` is a
// bit set of 1 = f, 2 = grad, 4 = hessian (interp) / 1 = f, 2 = grad (spread).
// launch_interp / launch_spread return the ConvKernel family they launched.
enum ConvKernel { CONV_NONE = 0, CONV_GROUP = 1, CONV_TILE = 2, CONV_LINE = 3, CONV_GENERIC = 4 };
void bin_nodes(const ConvArgs &a, bool fp32, cudaStream_t s);
int launch_interp(const ConvArgs &a, int mode, bool fp32, cudaStream_t s);
int launch_spread(const ConvArgs &a, int mode, bool fp32, cudaStream_t s);
// Kernel families behind launch_interp / launch_spread; each returns false
// when it has no instance for the cutoff or mode.
// FP32-mixed f-only interpolation on a BIN_LINE binning (interp_line.cu)
bool launch_interp_line(const ConvArgs &a, cudaStream_t s);
// FP32-mixed interpolation with the gradient (mode 2 or 3) on a BIN_LINE binning (interp_line_g.cu)
bool launch_interp_line_g(const ConvArgs &a, int mode, cudaStream_t s);
// FP32-mixed f-only interpolation on a BIN_GROUP binning (interp_group.cu)
bool launch_interp_group(const ConvArgs &a, cudaStream_t s);
// one warp per node on tile binnings (interp_tile_f32.cu, interp_tile_f64.cu)
bool launch_interp_tile_f32(const ConvArgs &a, int mode, cudaStream_t s);
bool launch_interp_tile_f64(const ConvArgs &a, int mode, cudaStream_t s);
// FP32-mixed f-only spreading on a BIN_LINE binning (spread_line_f.cu)
bool launch_spread_line_f(const ConvArgs &a, cudaStream_t s);
// the same kernels of one cutoff over the items of a MultiConv (first[n] blocks)
bool launch_interp_line_multi(const MultiConv &mc, int cut, cudaStream_t s);
bool launch_spread_line_f_multi(const MultiConv &mc, int cut, cudaStream_t s);
// whether launch_interp / launch_spread would take k_interp_line /
// k_spread_line_f for these arguments
bool interp_line_chosen(const ConvArgs &a, int mode, bool fp32);
bool spread_line_f_chosen(const ConvArgs &a, int mode, bool fp32);
// copies `a` to device memory `dst` in stream order (a kernel with `a` as its
// parameter, so that graph replays write the captured arguments)
void store_conv_args(const ConvArgs &a, ConvArgs *dst, cudaStream_t s);
// lines of tiles (spread_line_f32.cu, spread_line_f64.cu)
bool launch_spread_line_f32(const ConvArgs &a, int mode, cudaStream_t s);
bool launch_spread_line_f64(const ConvArgs &a, int mode, cudaStream_t s);
// one thread per node, any cutoff (generic.cu)
void launch_interp_generic(const ConvArgs &a, int mode, bool fp32, cudaStream_t s);
void launch_spread_generic(const ConvArgs &a, int mode, bool fp32, cudaStream_t s);
// Tile shape and BinMode of the binning for interpolation (spread = false)
// or spreading (spread = true); f_only: the interpolation computes f alone
// (no gradient or Hessian in the same pass); method: the plan's conv method.
void choose_tiles(int cut, bool fp32, bool spread, bool f_only, int method, const int *n, int64_t M, int *T,
                  int *line_mode);

// Deconvolution (deconv.cu).
struct DeconvArgs {
  int N[3], n[3];
  int64_t Nl[3], ks[3];  // stored block of f_hat (c2r: Nl2 = N2/2+1)
  int transposed, c2r;
  const double *inv[3];  // inv_phi_hat per axis for k = ks..ks+Nl-1
  double scale;          // power of two undoing the FP32 window scaling (1 in FP64)
  int interlaced;
  int ik;                // 0 none, 1 gradient component ik_dim, 2 Hessian component ik_dim
  int ik_dim;
  const double *fhat_in; // trafo: f_hat (complex double)
  double *fhat_out;      // adjoint: accumulated f_hat
  void *grid;            // n0*n1*n2 complex, compute precision
};
void launch_deconv_pad(const DeconvArgs &a, bool fp32, cudaStream_t s);
void launch_deconv_crop_acc(const DeconvArgs &a, bool fp32, cudaStream_t s);

// Verification helpers and the direct NDFT (sort.cu, ndft.cu).
void launch_node_index(const double *x, int64_t M, const int *n, int m, int il, bool integer_path, long long *u,
                       cudaStream_t s);
int radix_sort_nodes(const double *x, int64_t M, const int *n, int m, long long *pairs_dev, cudaStream_t s);

struct NdftArgs {
  int N[3];
  int64_t Nl[3], ks[3];
  int transposed, c2r;
  int64_t M;
  const double *x;
  const double *fhat;  // complex
  double *f, *grad, *hess;
  const double *f_in, *grad_in;
  double *fhat_out;
  unsigned cflags;
};
void launch_ndft_trafo(const NdftArgs &a, cudaStream_t s);
void launch_ndft_adj(const NdftArgs &a, cudaStream_t s);

}  // namespace pg
