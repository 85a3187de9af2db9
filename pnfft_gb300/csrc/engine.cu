// engine.cu -- device side of pnfft_trafo / pnfft_adj: buffers, cuFFT plans,
// stage timing, and the orchestration of api/api-basic.c:100-378 on one GPU.
//
//   trafo: [bin nodes] -> D (+pad) -> FFT -> B          (api-basic.c:170-196)
//          DIFF_IK: one D/FFT/B pass per output component (100-167)
//          INTERLACED: a second, shifted pass, each scaled by 1/2 (233-240)
//   adj:   [bin nodes] -> B^T -> FFT^H -> D^T (+crop)   (307-333)
//          DIFF_IK: one B^T/FFT^H/D^T pass per input component (249-305)
// The PFFT transposes and ghost-cell exchanges of the reference have no
// counterpart: the grid is one n0 x n1 x n2 array in HBM.
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdio.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <unordered_set>

#include "pg_internal.h"
#include "pg_kernels.h"

namespace pg {

#define PG_CUDA(call)                                                                             \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) {                                                                      \
      set_error("CUDA error %s at %s:%d: %s", cudaGetErrorName(e_), __FILE__, __LINE__,           \
                cudaGetErrorString(e_));                                                          \
      return -1;                                                                                  \
    }                                                                                             \
  } while (0)

#define PG_FFT(call)                                                                              \
  do {                                                                                            \
    cufftResult r_ = (call);                                                                      \
    if (r_ != CUFFT_SUCCESS) {                                                                    \
      set_error("cuFFT error %d at %s:%d", (int)r_, __FILE__, __LINE__);                         \
      return -1;                                                                                  \
    }                                                                                             \
  } while (0)

static const unsigned C_F = PNFFT_COMPUTE_F, C_GRAD = PNFFT_COMPUTE_GRAD_F, C_HESS = PNFFT_COMPUTE_HESSIAN_F;

struct Stage {
  int idx;  // PNFFT_TIMER_*
  int adj;
  cudaEvent_t a, b;
};

struct DevState {
  int device = -1;
  cudaStream_t own = nullptr, stream = nullptr;
  // the trafo bins its nodes on `aux` while D and the FFT run on `stream`
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  void *grid = nullptr;
  size_t grid_bytes = 0;
  cufftHandle fft = 0;
  int fft_prec = -1;
  double *inv[3] = {nullptr, nullptr, nullptr};
  void *tab[3][3] = {{nullptr}};
  float *poly = nullptr;  // fitted FP32 window polynomials (nullptr: use the formula), then their pairs
  size_t poly_rows = 0;   // floats of the rows (the pairs follow)
  int poly_ncoef = kPolyCoef;  // coefficients used of each row (12 or 16)
  uint64_t tables_for = ~0ull;
  double *fhat = nullptr;
  size_t fhat_cap = 0;
  std::vector<Stage> pending;
  bool capturing = false;  // the current call is being captured into a CUDA graph
  std::vector<cudaEvent_t> free_ev;
  // batched convolutions (pnfft_gb300_batch_begin / _end): the k-th deferred
  // call of this plan in an open batch uses grid bgrid[k] and keeps its
  // arguments in bargs[k]; both stay allocated for later batches and graph
  // replays
  std::vector<void *> bgrid;
  std::vector<ConvArgs *> bargs;
  std::vector<cudaEvent_t> bev;  // recorded on the call's stream once its part before B / B^T is issued
  int bslot = 0;  // deferred calls of this plan in the open batch
};

// A binning of a node set onto grid tiles, kept with the node set: one slot
// per layout (0: lines of 4x4x4 tiles, which serve B and B^T alike; 1: the
// 8x8x8 tiles of conv methods 2 and 3) and interlacing pass.  A binning of
// fixed nodes is reused by every later call with the same plan, precision and
// coordinates, in either direction.
struct BinSlot {
  Binning b = {};
  int64_t cap = 0;
  int T[3] = {0, 0, 0};
  int line_mode = 0;
  int prec = -1;
  uint64_t plan = 0, ver = 0;  // plan uid and node version of the binned nodes
  bool valid = false;
};

struct NodeDev {
  double *x = nullptr, *f = nullptr, *grad = nullptr, *hess = nullptr;
  int64_t cap = 0;
  // the device copy of x matches the host x of this version (fixed nodes only)
  bool x_valid = false;
  uint64_t x_ver = 0;
  BinSlot bins[2][2];  // [layout][plain | interlaced pass], allocated on first use
};

// ---------------------------------------------------------------------------
// host memory of pnfft_malloc: page-locked when a device is present
// ---------------------------------------------------------------------------
static std::mutex g_pin_mu;
static std::unordered_set<void *> g_pinned;

int engine_device_count() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

void *engine_host_alloc(size_t bytes) {
  if (bytes == 0) return nullptr;
  void *p = nullptr;
  if (engine_device_count() > 0 && cudaMallocHost(&p, bytes) == cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    g_pinned.insert(p);
    return p;
  }
  cudaGetLastError();
  return nullptr;
}

bool engine_host_free(void *p) {
  {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto it = g_pinned.find(p);
    if (it == g_pinned.end()) return false;
    g_pinned.erase(it);
  }
  cudaFreeHost(p);
  return true;
}

// ---------------------------------------------------------------------------
// device state
// ---------------------------------------------------------------------------
static int ensure_dev(pnfft_plan p) {
  if (!p->dev) p->dev = new DevState();
  DevState *d = p->dev;
  if (d->device < 0) {
    int n = engine_device_count();
    if (n <= 0) {
      set_error("libpnfft_gb300: no CUDA device is visible; this library has no CPU path");
      return -1;
    }
    PG_CUDA(cudaGetDevice(&d->device));
    PG_CUDA(cudaStreamCreateWithFlags(&d->own, cudaStreamNonBlocking));
    PG_CUDA(cudaStreamCreateWithFlags(&d->aux, cudaStreamNonBlocking));
    PG_CUDA(cudaEventCreateWithFlags(&d->ev_fork, cudaEventDisableTiming));
    PG_CUDA(cudaEventCreateWithFlags(&d->ev_join, cudaEventDisableTiming));
  }
  d->stream = p->user_stream ? (cudaStream_t)p->user_stream : d->own;
  return 0;
}

static bool fp32(pnfft_plan p) { return p->precision == PNFFT_GB300_FP32_MIXED; }
static size_t celem(pnfft_plan p) { return fp32(p) ? 8 : 16; }

static int ensure_grid_fft(pnfft_plan p) {
  DevState *d = p->dev;
  size_t bytes = (size_t)p->n[0] * p->n[1] * p->n[2] * celem(p);
  if (d->grid_bytes < bytes) {
    if (d->grid) cudaFree(d->grid);
    d->grid = nullptr;
    d->grid_bytes = 0;
    PG_CUDA(cudaMalloc(&d->grid, bytes));
    d->grid_bytes = bytes;
  }
  if (d->fft_prec != p->precision) {
    if (d->fft_prec >= 0) cufftDestroy(d->fft);
    d->fft_prec = -1;
    PG_FFT(cufftPlan3d(&d->fft, (int)p->n[0], (int)p->n[1], (int)p->n[2], fp32(p) ? CUFFT_C2C : CUFFT_Z2Z));
    d->fft_prec = p->precision;
  }
  PG_FFT(cufftSetStream(d->fft, d->stream));
  return 0;
}

// FP32-mixed plans return the window of axis t times 2^-k with 2^k <= psi(0)
// (psi(0) < 2 needs no scaling); D is multiplied by 2^(k0+k1+k2).
static int window_kscale(pnfft_plan p, int t) {
  if (!fp32(p)) return 0;
  double out[3];
  window_eval<double>(p->window, p->m, (double)p->n[t], p->b[t], 0.0, (double)p->m, 0, out);
  return (out[0] >= 2.0) ? (int)floor(log2(out[0])) : 0;
}

// Polynomial fits of the window on each cell, for the FP32-mixed kernels.
// Every window is an entire function of y on each unit cell (Kaiser-Bessel
// and Bessel-I0 through sinh(sqrt z)/sqrt z and I0(sqrt z) with z = b^2 (m^2 -
// y^2), the B-spline a polynomial of degree 2m-1), so Chebyshev interpolation
// at ncoef points (degree ncoef - 1) converges fast; the fit is converted to
// the monomial basis in u = dist - 1/2 and rounded to float, in rows of
// kPolyCoef with zeros above ncoef.  The fit is kept only if, on 64 points
// per cell, it matches the FP64 formula to 1e-8 of the largest value of each
// derivative order (else the kernels evaluate the formula).  Derivatives
// come from the formula (psi', psi'' in x units).
static bool fit_window_poly(pnfft_plan p, std::vector<float> &out, int ncoef) {
  const int cut = p->cutoff, P = ncoef - 1;
  out.assign((size_t)3 * 3 * cut * kPolyCoef, 0.f);
  std::vector<double> f(ncoef), c(ncoef), mono(ncoef), tkm1(ncoef), tk(ncoef), tn(ncoef);
  for (int t = 0; t < 3; t++) {
    const double n = (double)p->n[t], b = p->b[t];
    const double sc = ldexp(1.0, -window_kscale(p, t));
    for (int der = 0; der <= 2; der++) {
      double vmax = 0.0, emax = 0.0;
      for (int s = 0; s < cut; s++) {
        for (int j = 0; j < ncoef; j++) {
          const double d = 0.5 + 0.5 * cos(kPi * (j + 0.5) / ncoef);
          double o[3];
          window_eval<double>(p->window, p->m, n, b, d + (double)(p->m - s), (double)s - d, der, o);
          f[j] = o[der];
        }
        for (int k = 0; k < ncoef; k++) {
          double sum = 0.0;
          for (int j = 0; j < ncoef; j++) sum += f[j] * cos(kPi * k * (j + 0.5) / ncoef);
          c[k] = 2.0 * sum / ncoef;
        }
        c[0] *= 0.5;
        // sum_k c_k T_k(v), v = 2u, in monomials of v
        std::fill(mono.begin(), mono.end(), 0.0);
        std::fill(tkm1.begin(), tkm1.end(), 0.0);
        std::fill(tk.begin(), tk.end(), 0.0);
        tkm1[0] = 1.0;
        tk[1] = 1.0;
        mono[0] = c[0];
        mono[1] = c[1];
        for (int k = 2; k <= P; k++) {
          for (int i = 0; i < ncoef; i++) tn[i] = (i > 0 ? 2.0 * tk[i - 1] : 0.0) - tkm1[i];
          for (int i = 0; i < ncoef; i++) mono[i] += c[k] * tn[i];
          tkm1 = tk;
          tk = tn;
        }
        float *row = &out[((size_t)(der * 3 + t) * cut + s) * kPolyCoef];
        for (int i = 0; i < ncoef; i++) {
          mono[i] *= ldexp(1.0, i) * sc;
          row[i] = (float)mono[i];
        }
        // the approximation error of the fit (FP64 coefficients); rounding
        // them to float adds the FP32 evaluation error of any method
        for (int q = 0; q < 64; q++) {
          const double d = (q + 0.5) / 64.0, u = d - 0.5;
          double o[3];
          window_eval<double>(p->window, p->m, n, b, d + (double)(p->m - s), (double)s - d, der, o);
          double h = 0.0;
          for (int i = P; i >= 0; i--) h = h * u + mono[i];
          vmax = std::max(vmax, fabs(o[der] * sc));
          emax = std::max(emax, fabs(h - o[der] * sc));
        }
      }
      if (!(emax <= 1e-8 * vmax + 1e-300)) return false;
    }
  }
  return true;
}

static int ensure_tables(pnfft_plan p) {
  DevState *d = p->dev;
  uint64_t want = (p->table_version << 1) | (uint64_t)(fp32(p) ? 1 : 0);
  if (d->tables_for == want) return 0;
  for (int t = 0; t < 3; t++) {
    if (d->inv[t]) cudaFree(d->inv[t]);
    d->inv[t] = nullptr;
    size_t nb = sizeof(double) * p->inv[t].size();
    PG_CUDA(cudaMalloc(&d->inv[t], nb > 0 ? nb : 8));
    PG_CUDA(cudaMemcpy(d->inv[t], p->inv[t].data(), nb, cudaMemcpyHostToDevice));
  }
  for (int der = 0; der < 3; der++)
    for (int t = 0; t < 3; t++) {
      if (d->tab[der][t]) cudaFree(d->tab[der][t]);
      d->tab[der][t] = nullptr;
      const std::vector<double> &h = p->tab[der][t];
      if (h.empty()) continue;
      if (fp32(p)) {
        std::vector<float> tmp(h.size());
        const int ks = window_kscale(p, t);
        for (size_t i = 0; i < h.size(); i++) tmp[i] = (float)ldexp(h[i], -ks);
        PG_CUDA(cudaMalloc(&d->tab[der][t], sizeof(float) * tmp.size()));
        PG_CUDA(cudaMemcpy(d->tab[der][t], tmp.data(), sizeof(float) * tmp.size(), cudaMemcpyHostToDevice));
      } else {
        PG_CUDA(cudaMalloc(&d->tab[der][t], sizeof(double) * h.size()));
        PG_CUDA(cudaMemcpy(d->tab[der][t], h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
      }
    }
  if (d->poly) cudaFree(d->poly);
  d->poly = nullptr;
  d->poly_ncoef = kPolyCoef;
  if (fp32(p) && p->intpol_order < 0) {
    // the shortest fit that meets the tolerance: 12 coefficients, else 16
    std::vector<float> h;
    for (int nc : {12, kPolyCoef}) {
      if (fit_window_poly(p, h, nc)) {
        // the rows, then the same coefficients in pairs of stencil points
        const int cut = p->cutoff, np = (cut + 1) / 2;
        d->poly_rows = h.size();
        h.resize(d->poly_rows + (size_t)9 * np * 32, 0.f);
        float *pp = h.data() + d->poly_rows;
        for (int r = 0; r < 9; r++)
          for (int cp = 0; cp < np; cp++)
            for (int k = 0; k < kPolyCoef; k++)
              for (int l = 0; l < 2; l++)
                if (2 * cp + l < cut) pp[((r * np + cp) * 16 + k) * 2 + l] = h[(size_t)(r * cut + 2 * cp + l) * kPolyCoef + k];
        PG_CUDA(cudaMalloc(&d->poly, sizeof(float) * h.size()));
        PG_CUDA(cudaMemcpy(d->poly, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice));
        d->poly_ncoef = nc;
        break;
      }
    }
  }
  d->tables_for = want;
  return 0;
}

static void free_binning(Binning &b) {
  int **arrs[] = {&b.key,       &b.perm,    &b.count,    &b.start,      &b.rank,      &b.nsub_tile, &b.sub_off,
                  &b.sub_tile,  &b.sub_first, &b.sub_cnt, &b.nsub,      &b.tsub_tile, &b.tsub_first, &b.tsub_cnt,
                  &b.ntsub};
  for (int **a : arrs) {
    if (*a) cudaFree(*a);
    *a = nullptr;
  }
  if (b.rec) cudaFree(b.rec);
  if (b.rec_tmp) cudaFree(b.rec_tmp);
  if (b.bsum) cudaFree(b.bsum);
  b.rec = b.rec_tmp = nullptr;
  b.bsum = nullptr;
}

static NodeDev *node_dev(pnfft_nodes nd) {
  if (!nd->dev) nd->dev = new NodeDev();
  return nd->dev;
}

// ---------------------------------------------------------------------------
// batched convolutions
//
// Between pnfft_gb300_batch_begin(stream) and pnfft_gb300_batch_end(), a call
// (on any stream) with device arrays, fixed nodes and an FP32-mixed f-only
// line convolution (no ik, interlacing, gradient or Hessian) too small to
// fill the GPU alone runs its binning
// and D + F (trafo) or its binning and grid clearing (adjoint) at once into a
// grid of its own, and defers B or B^T.  The end of the batch waits on the
// batch stream for the deferred calls (an event per call), launches one kernel
// per direction and cutoff over the line sub-problems of all deferred calls
// (up to kMultiItems per launch), then the adjoints' F^H and D^T.  The
// calls of a batch must be independent (none reads what another writes).
// ---------------------------------------------------------------------------
struct Deferred {
  pnfft_plan p;
  BinSlot *slot;          // the node set's binning the call reads
  int adjoint, cut, max_subs;
  const ConvArgs *dargs;  // the call's arguments in device memory
  void *grid;
  cudaEvent_t ev;         // the batch stream waits for it before the batched launch
  DeconvArgs da;          // adjoint: D^T after F^H on `grid`
};

struct BatchState {
  bool active = false;
  cudaStream_t s = nullptr;
  std::vector<Deferred> items;
  std::vector<pnfft_plan> plans;  // plans with deferred calls
  int deferred = 0;               // calls deferred since the batch opened
  int launches = 0;               // batched kernel launches since the batch opened
  int last_deferred = 0, last_launches = 0;  // of the last closed batch
  cudaEvent_t ev = nullptr;       // orders a rebinning after an early flush
};
static BatchState g_batch;

static int fft_exec_on(pnfft_plan p, void *grid, int direction) {
  DevState *d = p->dev;
  if (fp32(p)) PG_FFT(cufftExecC2C(d->fft, (cufftComplex *)grid, (cufftComplex *)grid, direction));
  else PG_FFT(cufftExecZ2Z(d->fft, (cufftDoubleComplex *)grid, (cufftDoubleComplex *)grid, direction));
  return 0;
}

// Only calls too small to fill the GPU alone are deferred (fewer line
// sub-problems than 4 CTAs per SM): a large call keeps D, F and B back to
// back on one grid, which stays in L2, and fills the GPU by itself.
static bool batch_small(const Binning &b) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
  }
  return b.max_subs < 4 * sms;
}

// the grid and argument slot of the plan's next deferred call; false (the
// call then runs as usual) where a slot would need an allocation during a
// stream capture or the allocation fails
static bool batch_slot(pnfft_plan p, void **grid, ConvArgs **dargs, cudaEvent_t *ev) {
  DevState *d = p->dev;
  const int k = d->bslot;
  if (k >= (int)d->bgrid.size()) {
    if (d->capturing) return false;
    void *g = nullptr;
    ConvArgs *a = nullptr;
    cudaEvent_t e = nullptr;
    if (cudaMalloc(&g, d->grid_bytes) != cudaSuccess || cudaMalloc(&a, sizeof(ConvArgs)) != cudaSuccess ||
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      if (g) cudaFree(g);
      if (a) cudaFree(a);
      return false;
    }
    d->bgrid.push_back(g);
    d->bargs.push_back(a);
    d->bev.push_back(e);
  }
  *grid = d->bgrid[k];
  *dargs = d->bargs[k];
  *ev = d->bev[k];
  if (d->bslot++ == 0) g_batch.plans.push_back(p);
  return true;
}

static int batch_flush() {
  if (g_batch.items.empty()) return 0;
  const cudaStream_t s = g_batch.s;
  std::vector<Deferred> &items = g_batch.items;
  for (const Deferred &it : items) PG_CUDA(cudaStreamWaitEvent(s, it.ev, 0));
  for (int adj = 0; adj < 2; adj++) {
    std::vector<int> cuts;
    for (const Deferred &it : items)
      if (it.adjoint == adj && std::find(cuts.begin(), cuts.end(), it.cut) == cuts.end()) cuts.push_back(it.cut);
    for (int cut : cuts) {
      MultiConv mc;
      memset(&mc, 0, sizeof(mc));
      auto launch = [&]() -> bool {
        const bool ok = adj ? launch_spread_line_f_multi(mc, cut, s) : launch_interp_line_multi(mc, cut, s);
        g_batch.launches++;
        mc.n = 0;
        mc.first[0] = 0;
        return ok;
      };
      for (const Deferred &it : items) {
        if (it.adjoint != adj || it.cut != cut) continue;
        mc.args[mc.n] = it.dargs;
        mc.first[mc.n + 1] = mc.first[mc.n] + it.max_subs;
        mc.n++;
        if (mc.n == kMultiItems && !launch()) return set_error("batched convolution: no kernel for cutoff %d", cut), -1;
      }
      if (mc.n > 0 && !launch()) return set_error("batched convolution: no kernel for cutoff %d", cut), -1;
    }
  }
  for (const Deferred &it : items) {
    if (!it.adjoint) continue;
    DevState *d = it.p->dev;
    // the plan's FFT (and its work area) on the batch stream: after the work
    // already on the plan's stream, and before what follows there
    if (d->stream != s) {
      PG_CUDA(cudaEventRecord(d->ev_fork, d->stream));
      PG_CUDA(cudaStreamWaitEvent(s, d->ev_fork, 0));
    }
    PG_FFT(cufftSetStream(d->fft, s));
    const int rc = fft_exec_on(it.p, it.grid, CUFFT_INVERSE);
    PG_FFT(cufftSetStream(d->fft, d->stream));
    if (rc) return -1;
    launch_deconv_crop_acc(it.da, fp32(it.p), s);
    if (d->stream != s) {
      PG_CUDA(cudaEventRecord(d->ev_join, s));
      PG_CUDA(cudaStreamWaitEvent(d->stream, d->ev_join, 0));
    }
  }
  PG_CUDA(cudaGetLastError());
  for (pnfft_plan p : g_batch.plans)
    if (p->dev) p->dev->bslot = 0;
  items.clear();
  g_batch.plans.clear();
  return 0;
}

int engine_batch_begin(void *stream) {
  if (g_batch.active) return set_error("pnfft_gb300_batch_begin: a batch is already open"), -1;
  if (!stream) return set_error("pnfft_gb300_batch_begin: a stream is required"), -1;
  g_batch.active = true;
  g_batch.s = (cudaStream_t)stream;
  g_batch.deferred = g_batch.launches = 0;
  g_batch.items.clear();
  g_batch.plans.clear();
  return 0;
}

int engine_batch_end() {
  if (!g_batch.active) return set_error("pnfft_gb300_batch_end: no batch is open"), -1;
  const int rc = batch_flush();
  g_batch.active = false;
  g_batch.last_deferred = g_batch.deferred;
  g_batch.last_launches = g_batch.launches;
  g_batch.items.clear();
  for (pnfft_plan p : g_batch.plans)
    if (p->dev) p->dev->bslot = 0;
  g_batch.plans.clear();
  return rc;
}

void engine_batch_stats(int *deferred, int *launches) {
  *deferred = g_batch.last_deferred;
  *launches = g_batch.last_launches;
}

static bool batch_uses_slot(const BinSlot *sl) {
  for (const Deferred &it : g_batch.items)
    if (it.slot == sl) return true;
  return false;
}

// the binning slot of these nodes for pass `il` of a B (spread = 0) or B^T
// (spread = 1), (re)allocated for the plan's tile shape when needed
// the slot a binning of these nodes goes to, and whether its allocation
// already fits the plan's tile shape, sub-problem size and precision
static BinSlot *binning_target(pnfft_plan p, pnfft_nodes nd, int spread, int il, bool f_only, int *T,
                               int *line_mode, int *sub_max, bool *fits) {
  const int64_t M = nd->local_M;
  int n[3] = {(int)p->n[0], (int)p->n[1], (int)p->n[2]};
  choose_tiles(p->cutoff, fp32(p), spread != 0, f_only, p->conv_method[spread ? 1 : 0], n, M, T, line_mode);
  BinSlot &sl = node_dev(nd)->bins[*line_mode == BIN_LINE ? 0 : 1][il];
  *sub_max = *line_mode == BIN_LINE ? p->line_sub_max : 1024;
  bool same = T[0] == sl.T[0] && T[1] == sl.T[1] && T[2] == sl.T[2] && *line_mode == sl.line_mode &&
              sl.b.sub_max == *sub_max;
  for (int t = 0; t < 3; t++) same = same && sl.b.ntile[t] == (n[t] + T[t] - 1) / T[t];
  *fits = same && sl.cap >= M && sl.b.key && sl.prec == p->precision;
  return &sl;
}

static BinSlot *ensure_binning(pnfft_plan p, pnfft_nodes nd, int spread, int il, bool f_only) {
  const int64_t M = nd->local_M;
  int n[3] = {(int)p->n[0], (int)p->n[1], (int)p->n[2]};
  int T[3], line_mode = 0, sub_max = 0;
  bool fits = false;
  BinSlot &sl = *binning_target(p, nd, spread, il, f_only, T, &line_mode, &sub_max, &fits);
  if (fits) return &sl;
  int64_t cap = std::max<int64_t>(M, std::max<int64_t>(sl.cap, 1));
  Binning &b = sl.b;
  free_binning(b);
  sl.valid = false;
  for (int t = 0; t < 3; t++) {
    b.T[t] = T[t];
    b.ntile[t] = (n[t] + T[t] - 1) / T[t];
  }
  b.ntiles = b.ntile[0] * b.ntile[1] * b.ntile[2];
  b.line_mode = line_mode;
  b.nkeys = line_mode == BIN_GROUP ? b.ntiles * kBlocksPerTile : b.ntiles;
  // line binnings: at most line_sub_max nodes of a line per CTA (512 unless
  // tuned): dense clusters put thousands of nodes on a few lines, which would
  // otherwise run long after the others
  b.sub_max = sub_max;
  const int units = line_mode == BIN_LINE ? b.ntile[0] * b.ntile[1] : b.ntiles;
  b.max_subs = (int)(units + cap / b.sub_max + 1);
  b.max_tsubs = line_mode == BIN_LINE ? (int)(b.ntiles + cap / b.sub_max + 1) : 0;
  auto alloc = [&](int **ptr, size_t count) -> bool {
    if (cudaMalloc(ptr, sizeof(int) * std::max<size_t>(count, 1)) != cudaSuccess) {
      set_error("device allocation of the node binning failed (%zu ints)", count);
      return false;
    }
    return true;
  };
  const size_t recb = fp32(p) ? sizeof(float4) : sizeof(double4);
  if (!alloc(&b.key, cap) || !alloc(&b.perm, cap) || !alloc(&b.count, b.nkeys) || !alloc(&b.start, b.nkeys) ||
      !alloc(&b.rank, cap) || !alloc(&b.nsub_tile, b.nkeys) || !alloc(&b.sub_off, b.nkeys) ||
      !alloc(&b.sub_tile, b.max_subs) || !alloc(&b.sub_first, b.max_subs) || !alloc(&b.sub_cnt, b.max_subs) ||
      !alloc(&b.nsub, 2) || !alloc(&b.bsum, 2 * ((b.nkeys + 2047) / 2048 + 1)) ||
      (line_mode == BIN_LINE && (!alloc(&b.tsub_tile, b.max_tsubs) || !alloc(&b.tsub_first, b.max_tsubs) ||
                                 !alloc(&b.tsub_cnt, b.max_tsubs) || !alloc(&b.ntsub, 1))) ||
      cudaMalloc(&b.rec, recb * cap) != cudaSuccess || cudaMalloc(&b.rec_tmp, recb * cap) != cudaSuccess) {
    cudaGetLastError();
    if (!last_error()[0]) set_error("device allocation of the node records failed");
    free_binning(b);
    sl.cap = 0;
    return nullptr;
  }
  sl.cap = cap;
  sl.prec = p->precision;
  sl.line_mode = line_mode;
  for (int t = 0; t < 3; t++) sl.T[t] = T[t];
  return &sl;
}

static int ensure_node_buffers(pnfft_plan p, pnfft_nodes nd, unsigned cflags) {
  if (!nd->dev) nd->dev = new NodeDev();
  NodeDev *v = nd->dev;
  int64_t M = nd->local_M;
  if (v->cap < M) {
    cudaFree(v->x);
    cudaFree(v->f);
    cudaFree(v->grad);
    cudaFree(v->hess);
    v->x = v->f = v->grad = v->hess = nullptr;
    v->cap = 0;
    v->x_valid = false;
    size_t m = (size_t)std::max<int64_t>(M, 1);
    PG_CUDA(cudaMalloc(&v->x, sizeof(double) * 3 * m));
    PG_CUDA(cudaMalloc(&v->f, sizeof(double) * 2 * m));
    v->cap = M;
  }
  size_t m = (size_t)std::max<int64_t>(v->cap, 1);
  if ((cflags & C_GRAD) && !v->grad) PG_CUDA(cudaMalloc(&v->grad, sizeof(double) * 6 * m));
  if ((cflags & C_HESS) && !v->hess) PG_CUDA(cudaMalloc(&v->hess, sizeof(double) * 12 * m));
  (void)p;
  return 0;
}

// ---------------------------------------------------------------------------
// stage timers (CUDA events on the plan's stream)
// ---------------------------------------------------------------------------
static cudaEvent_t get_event(DevState *d) {
  if (!d->free_ev.empty()) {
    cudaEvent_t e = d->free_ev.back();
    d->free_ev.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

struct StageScope {
  DevState *d;
  Stage st;
  cudaStream_t s;
  StageScope(DevState *d_, int idx, int adj, cudaStream_t s_ = nullptr) : d(d_), s(s_ ? s_ : d_->stream) {
    if (d->capturing) return;  // no stage timers inside a captured graph
    st.idx = idx;
    st.adj = adj;
    st.a = get_event(d);
    st.b = get_event(d);
    cudaEventRecord(st.a, s);
  }
  ~StageScope() {
    if (d->capturing) return;
    cudaEventRecord(st.b, s);
    d->pending.push_back(st);
  }
};

void engine_flush_timers(pnfft_plan p) {
  DevState *d = p->dev;
  if (!d || d->pending.empty()) return;
  cudaStreamSynchronize(d->stream);
  bool seen[2] = {false, false};
  for (const Stage &s : d->pending) {
    if (!seen[s.adj]) {
      for (int i = 0; i < PNFFT_TIMER_LENGTH; i++) p->last_ms[s.adj][i] = 0;
      seen[s.adj] = true;
    }
    float ms = 0;
    if (cudaEventElapsedTime(&ms, s.a, s.b) == cudaSuccess) {
      double *tm = s.adj ? p->timer_adj : p->timer_trafo;
      tm[s.idx] += ms * 1e-3;
      p->last_ms[s.adj][s.idx] += ms;
    }
    d->free_ev.push_back(s.a);
    d->free_ev.push_back(s.b);
  }
  cudaGetLastError();
  d->pending.clear();
}

// ---------------------------------------------------------------------------
// building blocks
// ---------------------------------------------------------------------------
static WindowArgs window_args(pnfft_plan p) {
  WindowArgs w;
  w.kind = p->window;
  w.m = p->m;
  w.cut = p->cutoff;
  for (int t = 0; t < 3; t++) {
    w.n[t] = (int)p->n[t];
    w.b[t] = p->b[t];
    const double b = p->b[t];
    WinF &c = w.wf[t];
    c.n = (float)p->n[t];
    c.b = (float)b;
    c.b_lo = (float)(b - (double)c.b);
    const double ib = (b != 0.0) ? 1.0 / b : 0.0, pb = (b != 0.0) ? kPi / b : 0.0;
    c.ib = (float)ib;
    c.ib_lo = (float)(ib - (double)c.ib);
    c.pb = (float)pb;
    c.pb_lo = (float)(pb - (double)c.pb);
    c.gnorm = (b > 0.0) ? (float)(1.0 / sqrt(kPi * b)) : 0.f;
    c.kscale = window_kscale(p, t);
    c.wsc = ldexpf(1.f, -c.kscale);
  }
  w.intpol_order = p->intpol_order;
  w.intpol_K = (int)p->intpol_K;
  for (int der = 0; der < 3; der++)
    for (int t = 0; t < 3; t++) w.tab[der][t] = p->dev->tab[der][t];
  w.poly = p->dev->poly;
  w.poly_ncoef = p->dev->poly_ncoef;
  w.poly_pp = p->dev->poly ? p->dev->poly + p->dev->poly_rows : nullptr;
  return w;
}

static DeconvArgs deconv_args(pnfft_plan p) {
  DeconvArgs a;
  memset(&a, 0, sizeof(a));
  for (int t = 0; t < 3; t++) {
    a.N[t] = (int)p->N[t];
    a.n[t] = (int)p->n[t];
    a.Nl[t] = p->local_N[t];
    a.ks[t] = p->local_N_start[t];
    a.inv[t] = p->dev->inv[t];
  }
  a.transposed = (p->pnfft_flags & PNFFT_TRANSPOSED_F_HAT) ? 1 : 0;
  a.c2r = p->c2r;
  a.grid = p->dev->grid;
  a.scale = ldexp(1.0, window_kscale(p, 0) + window_kscale(p, 1) + window_kscale(p, 2));
  return a;
}

static int fft_exec(pnfft_plan p, int direction) {
  DevState *d = p->dev;
  if (fp32(p)) PG_FFT(cufftExecC2C(d->fft, (cufftComplex *)d->grid, (cufftComplex *)d->grid, direction));
  else PG_FFT(cufftExecZ2Z(d->fft, (cufftDoubleComplex *)d->grid, (cufftDoubleComplex *)d->grid, direction));
  return 0;
}

// bins the nodes for pass `il` unless a valid binning of the same fixed nodes exists
static int do_binning(pnfft_plan p, pnfft_nodes nd, ConvArgs &a, int il, int adj, cudaStream_t s, bool f_only) {
  DevState *d = p->dev;
  if (!s) s = d->stream;
  if (!g_batch.items.empty()) {
    // a deferred call of the open batch reads this slot: run the batch before
    // the slot is reallocated or rebinned
    int T[3], lm = 0, sm = 0;
    bool fits = false;
    BinSlot *t = binning_target(p, nd, adj, il, f_only, T, &lm, &sm, &fits);
    const bool reuse = fits && nd->fixed && t->valid && t->plan == p->uid && t->ver == nd->version;
    if (!reuse && batch_uses_slot(t)) {
      if (batch_flush()) return -1;
      // the flushed kernels read the slot on the batch stream: the binning
      // below, on its own stream, waits for them
      if (!g_batch.ev) PG_CUDA(cudaEventCreateWithFlags(&g_batch.ev, cudaEventDisableTiming));
      PG_CUDA(cudaEventRecord(g_batch.ev, g_batch.s));
      PG_CUDA(cudaStreamWaitEvent(s, g_batch.ev, 0));
    }
  }
  BinSlot *sl = ensure_binning(p, nd, adj, il, f_only);
  if (!sl) return -1;
  a.bin = sl->b;
  const bool reuse = nd->fixed && sl->valid && sl->plan == p->uid && sl->ver == nd->version;
  if (!reuse) {
    StageScope sc(d, PNFFT_TIMER_SORT_NODES, adj, s);
    bin_nodes(a, fp32(p), s);
    sl->valid = true;
    sl->plan = p->uid;
    sl->ver = nd->version;
  }
  return 0;
}

struct Arrays {
  const double *x;
  double *f, *grad, *hess;  // node arrays on the device
  double *fhat;             // f_hat on the device
};

static int resolve_arrays(pnfft_plan p, pnfft_nodes nd, unsigned cflags, bool adjoint, Arrays &A, bool &zero_copy,
                          cudaStream_t xs = nullptr) {
  DevState *d = p->dev;
  if (!xs) xs = d->stream;
  int64_t M = nd ? nd->local_M : 0;
  const int tuple = p->c2r ? 1 : 2;
  zero_copy = nd && nd->u_x;
  if (nd) {
    if (zero_copy) {
      A.x = nd->u_x;
      A.f = (double *)nd->u_f;
      A.grad = (double *)nd->u_grad;
      A.hess = (double *)nd->u_hess;
    } else {
      if (ensure_node_buffers(p, nd, cflags)) return -1;
      NodeDev *v = nd->dev;
      A.x = v->x;
      A.f = v->f;
      A.grad = v->grad;
      A.hess = v->hess;
      if (M > 0) {
        if (!nd->x) {
          set_error("pnfft: nodes->x is not allocated");
          return -1;
        }
        if (!adjoint) {
          if ((cflags & C_F) && !nd->f) return set_error("pnfft_trafo: missing memory allocation of nodes->f"), -1;
          if ((cflags & C_GRAD) && !nd->grad_f)
            return set_error("pnfft_trafo: missing memory allocation of nodes->grad_f"), -1;
          if ((cflags & C_HESS) && !nd->hessian_f)
            return set_error("pnfft_trafo: missing memory allocation of nodes->hessian_f"), -1;
        }
        // fixed nodes (pnfft_precompute_psi / pnfft_gb300_nodes_set_fixed): the
        // coordinates are promised constant, so the device copy is reused
        if (!(nd->fixed && v->x_valid && v->x_ver == nd->version)) {
          PG_CUDA(cudaMemcpyAsync(v->x, nd->x, sizeof(double) * 3 * M, cudaMemcpyHostToDevice, xs));
          v->x_valid = true;
          v->x_ver = nd->version;
        }
        bool upload_out = !adjoint && (cflags & PNFFT_COMPUTE_ACCUMULATED);
        if ((cflags & C_F) && (adjoint || upload_out)) {
          if (!nd->f) {
            set_error("pnfft: missing memory allocation of nodes->f");
            return -1;
          }
          PG_CUDA(cudaMemcpyAsync(v->f, nd->f, sizeof(double) * tuple * M, cudaMemcpyHostToDevice, d->stream));
        }
        if ((cflags & C_GRAD) && (adjoint || upload_out)) {
          if (!nd->grad_f) {
            set_error("pnfft: missing memory allocation of nodes->grad_f");
            return -1;
          }
          PG_CUDA(cudaMemcpyAsync(v->grad, nd->grad_f, sizeof(double) * 3 * tuple * M, cudaMemcpyHostToDevice,
                                  d->stream));
        }
        if (!adjoint && (cflags & C_HESS) && upload_out) {
          if (!nd->hessian_f) {
            set_error("pnfft: missing memory allocation of nodes->hessian_f");
            return -1;
          }
          PG_CUDA(cudaMemcpyAsync(v->hess, nd->hessian_f, sizeof(double) * 6 * tuple * M, cudaMemcpyHostToDevice,
                                  d->stream));
        }
      }
    }
  } else {
    A.x = nullptr;
    A.f = A.grad = A.hess = nullptr;
  }
  // f_hat
  size_t fb = sizeof(double) * 2 * (size_t)p->local_N_total;
  if (p->d_f_hat_user) {
    A.fhat = (double *)p->d_f_hat_user;
  } else {
    if (d->fhat_cap < fb) {
      if (d->fhat) cudaFree(d->fhat);
      d->fhat = nullptr;
      d->fhat_cap = 0;
      PG_CUDA(cudaMalloc(&d->fhat, fb > 0 ? fb : 16));
      d->fhat_cap = fb;
    }
    A.fhat = d->fhat;
    bool need_in = !adjoint || (cflags & PNFFT_COMPUTE_ACCUMULATED);
    if (need_in && fb > 0) {
      if (!p->f_hat) {
        set_error("pnfft: f_hat is not allocated");
        return -1;
      }
      PG_CUDA(cudaMemcpyAsync(d->fhat, p->f_hat, fb, cudaMemcpyHostToDevice, d->stream));
    }
  }
  return 0;
}

// A call made while the plan's stream is being captured into a CUDA graph
// must touch device memory only: every array attached with
// pnfft_gb300_set_device_arrays / _set_device_f_hat, and the buffers already
// allocated by an earlier call with the same sizes.  Host arrays would need
// copies and a synchronisation, so they are refused.
static int begin_call(pnfft_plan p, pnfft_nodes nd, const char *who) {
  DevState *d = p->dev;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  PG_CUDA(cudaStreamIsCapturing(d->stream, &cs));
  d->capturing = cs != cudaStreamCaptureStatusNone;
  if (d->capturing && ((nd && !nd->u_x) || !p->d_f_hat_user)) {
    set_error("%s: the stream is being captured into a CUDA graph; attach device arrays for the nodes and f_hat "
              "(pnfft_gb300_set_device_arrays / pnfft_gb300_set_device_f_hat) and make one call before capturing",
              who);
    return -1;
  }
  return 0;
}

// Joins the auxiliary stream back into the plan's stream once it has been
// forked, on every way out of a call: an error return must not leave the
// upload of x or the binning running after the call (the caller may free or
// reuse the arrays), nor leave an unjoined fork in a stream capture.
struct ForkJoin {
  DevState *d;
  cudaStream_t s;
  bool pending = false;
  // the plan's stream waits for everything issued on the auxiliary stream so far
  cudaError_t join() {
    pending = false;
    cudaError_t e = cudaEventRecord(d->ev_join, d->aux);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, d->ev_join, 0);
    return e;
  }
  ~ForkJoin() {
    if (pending) join();
  }
};

// ---------------------------------------------------------------------------
// pnfft_trafo
// ---------------------------------------------------------------------------
int engine_trafo(pnfft_plan p, pnfft_nodes nd, unsigned cflags) {
  if (ensure_dev(p)) return -1;
  DevState *d = p->dev;
  cudaStream_t s = d->stream;
  if (begin_call(p, nd, "pnfft_trafo")) return -1;
  if (ensure_grid_fft(p) || ensure_tables(p)) return -1;
  int64_t M = nd ? nd->local_M : 0;
  const int tuple = p->c2r ? 1 : 2;
  Arrays A;
  bool zc = false;
  // the node work (copy of x, binning) runs on the auxiliary stream, forked
  // from the plan's stream, while D and F run; B waits for it
  const bool fork = nd && M > 0 && !(cflags & (PNFFT_OMIT_CONV | PNFFT_COMPUTE_DIRECT));
  cudaStream_t xs = fork ? d->aux : s;
  ForkJoin fj{d, s};
  if (fork) {
    PG_CUDA(cudaEventRecord(d->ev_fork, s));
    PG_CUDA(cudaStreamWaitEvent(d->aux, d->ev_fork, 0));
    fj.pending = true;
  }
  {
    StageScope whole(d, PNFFT_TIMER_WHOLE, 0);
    if (resolve_arrays(p, nd, cflags, false, A, zc, xs)) return -1;
    // zero the outputs (api-basic.c:210-222; trafo_A always overwrites, 400-414)
    bool zero = (!(cflags & PNFFT_COMPUTE_ACCUMULATED) && !(cflags & PNFFT_OMIT_CONV)) ||
                (cflags & PNFFT_COMPUTE_DIRECT);
    if (zero && M > 0) {
      if ((cflags & C_F) && A.f) PG_CUDA(cudaMemsetAsync(A.f, 0, sizeof(double) * tuple * M, s));
      if ((cflags & C_GRAD) && A.grad) PG_CUDA(cudaMemsetAsync(A.grad, 0, sizeof(double) * 3 * tuple * M, s));
      if ((cflags & C_HESS) && A.hess) PG_CUDA(cudaMemsetAsync(A.hess, 0, sizeof(double) * 6 * tuple * M, s));
    }
    if ((cflags & C_F) && M > 0 && !A.f) return set_error("pnfft_trafo: missing memory allocation of nodes->f"), -1;
    if ((cflags & C_GRAD) && M > 0 && !A.grad)
      return set_error("pnfft_trafo: missing memory allocation of nodes->grad_f"), -1;
    if ((cflags & C_HESS) && M > 0 && !A.hess)
      return set_error("pnfft_trafo: missing memory allocation of nodes->hessian_f"), -1;

    if (cflags & PNFFT_COMPUTE_DIRECT) {
      NdftArgs na;
      memset(&na, 0, sizeof(na));
      for (int t = 0; t < 3; t++) {
        na.N[t] = (int)p->N[t];
        na.Nl[t] = p->local_N[t];
        na.ks[t] = p->local_N_start[t];
      }
      na.transposed = (p->pnfft_flags & PNFFT_TRANSPOSED_F_HAT) ? 1 : 0;
      na.c2r = p->c2r;
      na.M = M;
      na.x = A.x;
      na.fhat = A.fhat;
      na.f = A.f;
      na.grad = A.grad;
      na.hess = A.hess;
      na.cflags = cflags;
      launch_ndft_trafo(na, s);
    } else {
      const bool il_plan = (p->pnfft_flags & PNFFT_INTERLACED) != 0;
      const bool ik = (p->pnfft_flags & PNFFT_DIFF_IK) != 0;
      const bool f32 = fp32(p);
      // every interpolation of this call computes f alone (ik: one pass per component)
      const bool f_only = ik || !(cflags & (C_GRAD | C_HESS));
      ConvArgs ca;
      memset(&ca, 0, sizeof(ca));
      ca.w = window_args(p);
      ca.generic = p->conv_method[0] == 1;
      ca.method = p->conv_method[0];
      ca.real_only = p->c2r || (p->pnfft_flags & PNFFT_PRE_QUAD_PSI) ? 1 : 0;
      ca.real_io = p->c2r;
      ca.M = M;
      ca.x = A.x;
      ca.grid = d->grid;
      DeconvArgs da = deconv_args(p);
      da.fhat_in = A.fhat;
      Binning pass_bin[2] = {};
      if (fork) {
        for (int pass = 0; pass < (il_plan ? 2 : 1); pass++) {
          ca.il = il_plan ? pass : 0;
          if (do_binning(p, nd, ca, ca.il, 0, d->aux, f_only)) return -1;
          pass_bin[pass] = ca.bin;
        }
      }
      // an open batch defers B: D and F go to the call's own grid
      void *bgrid = nullptr;
      ConvArgs *bdargs = nullptr;
      cudaEvent_t bev = nullptr;
      bool defer = false;
      if (g_batch.active && zc && fork && !il_plan && !ik && nd->fixed && (cflags & C_F) &&
          !(cflags & (C_GRAD | C_HESS | PNFFT_OMIT_CONV | PNFFT_OMIT_FFT | PNFFT_OMIT_DECONV))) {
        ConvArgs probe = ca;
        probe.bin = pass_bin[0];
        defer = interp_line_chosen(probe, 1, f32) && batch_small(probe.bin) &&
                batch_slot(p, &bgrid, &bdargs, &bev);
      }
      if (defer) {
        ca.grid = bgrid;
        da.grid = bgrid;
      }
      for (int pass = 0; pass < (il_plan ? 2 : 1); pass++) {
        const int il = il_plan ? pass : 0;
        ca.use_il = il_plan ? 1 : 0;
        ca.il = il;
        ca.accum = (pass > 0 || (cflags & PNFFT_COMPUTE_ACCUMULATED)) ? 1 : 0;
        da.interlaced = il;
        ca.bin = pass_bin[pass];
        auto one = [&](int ikmode, int ikdim, double *out, int64_t off, int64_t stride, int mode) -> int {
          {
            StageScope sc(d, PNFFT_TIMER_MATRIX_D, 0);
            da.ik = ikmode;
            da.ik_dim = ikdim;
            if (!(cflags & PNFFT_OMIT_DECONV)) launch_deconv_pad(da, f32, s);
          }
          {
            StageScope sc(d, PNFFT_TIMER_MATRIX_F, 0);
            if (!(cflags & PNFFT_OMIT_FFT) && fft_exec(p, CUFFT_FORWARD)) return -1;
          }
          if (!(cflags & PNFFT_OMIT_CONV) && nd) {
            if (fj.pending) PG_CUDA(fj.join());  // B needs the binning from the auxiliary stream
            StageScope sc(d, PNFFT_TIMER_MATRIX_B, 0);
            ConvArgs c = ca;
            c.offset = off;
            c.stride = stride;
            if (mode & 4) {
              c.hess_out = out;
              p->last_conv[0] = launch_interp(c, 4, f32, s);
            } else if (mode == 1) {
              c.f_out = out;
              p->last_conv[0] = launch_interp(c, 1, f32, s);
            }
          }
          return 0;
        };
        if (ik) {
          if ((cflags & C_F) && one(0, 0, A.f, 0, 1, 1)) return -1;
          if (cflags & C_GRAD)
            for (int dim = 0; dim < 3; dim++)
              if (one(1, dim, A.grad, dim, 3, 1)) return -1;
          if (cflags & C_HESS)
            for (int dim = 0; dim < 6; dim++)
              if (one(2, dim, A.hess, dim, 6, 1)) return -1;
        } else {
          {
            StageScope sc(d, PNFFT_TIMER_MATRIX_D, 0);
            da.ik = 0;
            if (!(cflags & PNFFT_OMIT_DECONV)) launch_deconv_pad(da, f32, s);
          }
          {
            StageScope sc(d, PNFFT_TIMER_MATRIX_F, 0);
            if (!(cflags & PNFFT_OMIT_FFT) &&
                (defer ? fft_exec_on(p, bgrid, CUFFT_FORWARD) : fft_exec(p, CUFFT_FORWARD)))
              return -1;
          }
          if (!(cflags & PNFFT_OMIT_CONV) && nd) {
            if (fj.pending) PG_CUDA(fj.join());
            StageScope sc(d, PNFFT_TIMER_MATRIX_B, 0);
            ConvArgs c = ca;
            c.offset = 0;
            c.stride = 1;
            c.f_out = A.f;
            c.grad_out = A.grad;
            c.hess_out = A.hess;
            if (defer) {
              store_conv_args(c, bdargs, s);
              PG_CUDA(cudaEventRecord(bev, s));
              Deferred it;
              memset(&it, 0, sizeof(it));
              it.p = p;
              it.slot = &node_dev(nd)->bins[0][0];
              it.adjoint = 0;
              it.cut = p->cutoff;
              it.max_subs = c.bin.max_subs;
              it.dargs = bdargs;
              it.grid = bgrid;
              it.ev = bev;
              g_batch.items.push_back(it);
              g_batch.deferred++;
              p->last_conv[0] = CONV_LINE;
            } else {
              int mode = ((cflags & C_F) ? 1 : 0) | ((cflags & C_GRAD) ? 2 : 0);
              if (mode) p->last_conv[0] = launch_interp(c, mode, f32, s);
              if (cflags & C_HESS) p->last_conv[0] = launch_interp(c, 4, f32, s);
            }
          }
        }
      }
    }
    if (fj.pending) PG_CUDA(fj.join());  // every path joins the fork
    if (!zc && M > 0) {
      if (cflags & C_F) PG_CUDA(cudaMemcpyAsync(nd->f, A.f, sizeof(double) * tuple * M, cudaMemcpyDeviceToHost, s));
      if (cflags & C_GRAD)
        PG_CUDA(cudaMemcpyAsync(nd->grad_f, A.grad, sizeof(double) * 3 * tuple * M, cudaMemcpyDeviceToHost, s));
      if (cflags & C_HESS)
        PG_CUDA(cudaMemcpyAsync(nd->hessian_f, A.hess, sizeof(double) * 6 * tuple * M, cudaMemcpyDeviceToHost, s));
    }
  }
  p->timer_trafo[PNFFT_TIMER_ITER] += 1;
  PG_CUDA(cudaGetLastError());
  if (!(zc || !nd) || !p->d_f_hat_user) {
    PG_CUDA(cudaStreamSynchronize(s));
    engine_flush_timers(p);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// pnfft_adj
// ---------------------------------------------------------------------------
int engine_adj(pnfft_plan p, pnfft_nodes nd, unsigned cflags) {
  if (ensure_dev(p)) return -1;
  DevState *d = p->dev;
  cudaStream_t s = d->stream;
  if (begin_call(p, nd, "pnfft_adj")) return -1;
  if (ensure_grid_fft(p) || ensure_tables(p)) return -1;
  int64_t M = nd ? nd->local_M : 0;
  Arrays A;
  bool zc = false;
  size_t fb = sizeof(double) * 2 * (size_t)p->local_N_total;
  // as in the trafo: the copy of x and the binning run on the auxiliary
  // stream while the plan's stream uploads f and clears f_hat and the grid
  const bool fork = nd && M > 0 && !(cflags & (PNFFT_OMIT_CONV | PNFFT_COMPUTE_DIRECT));
  ForkJoin fj{d, s};
  if (fork) {
    PG_CUDA(cudaEventRecord(d->ev_fork, s));
    PG_CUDA(cudaStreamWaitEvent(d->aux, d->ev_fork, 0));
    fj.pending = true;
  }
  {
    StageScope whole(d, PNFFT_TIMER_WHOLE, 1);
    if (resolve_arrays(p, nd, cflags, true, A, zc, fork ? d->aux : s)) return -1;
    if (!(cflags & PNFFT_COMPUTE_ACCUMULATED) && fb > 0) PG_CUDA(cudaMemsetAsync(A.fhat, 0, fb, s));
    if ((cflags & C_F) && M > 0 && !A.f) return set_error("pnfft_adj: missing memory allocation of nodes->f"), -1;
    if ((cflags & C_GRAD) && M > 0 && !A.grad)
      return set_error("pnfft_adj: missing memory allocation of nodes->grad_f"), -1;

    if (cflags & PNFFT_COMPUTE_DIRECT) {
      NdftArgs na;
      memset(&na, 0, sizeof(na));
      for (int t = 0; t < 3; t++) {
        na.N[t] = (int)p->N[t];
        na.Nl[t] = p->local_N[t];
        na.ks[t] = p->local_N_start[t];
      }
      na.transposed = (p->pnfft_flags & PNFFT_TRANSPOSED_F_HAT) ? 1 : 0;
      na.c2r = p->c2r;
      na.M = M;
      na.x = A.x;
      na.f_in = A.f;
      na.grad_in = A.grad;
      na.fhat_out = A.fhat;
      na.cflags = cflags;
      launch_ndft_adj(na, s);
    } else {
      const bool il_plan = (p->pnfft_flags & PNFFT_INTERLACED) != 0;
      const bool ik = (p->pnfft_flags & PNFFT_DIFF_IK) != 0;
      const bool f32 = fp32(p);
      const size_t gbytes = (size_t)p->n[0] * p->n[1] * p->n[2] * celem(p);
      ConvArgs ca;
      memset(&ca, 0, sizeof(ca));
      ca.w = window_args(p);
      ca.generic = p->conv_method[1] == 1;
      ca.method = p->conv_method[1];
      ca.real_only = 0;
      ca.real_io = p->c2r;
      ca.M = M;
      ca.x = A.x;
      ca.grid = d->grid;
      DeconvArgs da = deconv_args(p);
      da.fhat_out = A.fhat;
      Binning pass_bin[2] = {};
      if (fork) {
        for (int pass = 0; pass < (il_plan ? 2 : 1); pass++) {
          ca.il = il_plan ? pass : 0;
          if (do_binning(p, nd, ca, ca.il, 1, d->aux, true)) return -1;
          pass_bin[pass] = ca.bin;
        }
      }
      // an open batch defers B^T, and F^H and D^T after it, on the call's own grid
      void *bgrid = nullptr;
      ConvArgs *bdargs = nullptr;
      cudaEvent_t bev = nullptr;
      bool defer = false;
      if (g_batch.active && zc && fork && !il_plan && !ik && nd->fixed && (cflags & C_F) &&
          !(cflags & (C_GRAD | PNFFT_OMIT_CONV | PNFFT_OMIT_FFT | PNFFT_OMIT_DECONV))) {
        ConvArgs probe = ca;
        probe.bin = pass_bin[0];
        defer = spread_line_f_chosen(probe, 1, f32) && batch_small(probe.bin) &&
                batch_slot(p, &bgrid, &bdargs, &bev);
      }
      for (int pass = 0; pass < (il_plan ? 2 : 1); pass++) {
        const int il = il_plan ? pass : 0;
        ca.use_il = il_plan ? 1 : 0;
        ca.il = il;
        da.interlaced = il;
        ca.bin = pass_bin[pass];
        auto one = [&](int ikmode, int ikdim, const double *fin, const double *gin, int64_t off, int64_t stride,
                       int mode) -> int {
          if (defer) {
            PG_CUDA(cudaMemsetAsync(bgrid, 0, gbytes, s));
            if (fj.pending) PG_CUDA(fj.join());
            ConvArgs c = ca;
            c.grid = bgrid;
            c.offset = off;
            c.stride = stride;
            c.f_in = fin;
            c.grad_in = gin;
            store_conv_args(c, bdargs, s);
            PG_CUDA(cudaEventRecord(bev, s));
            Deferred it;
            memset(&it, 0, sizeof(it));
            it.p = p;
            it.ev = bev;
            it.slot = &node_dev(nd)->bins[0][0];
            it.adjoint = 1;
            it.cut = p->cutoff;
            it.max_subs = c.bin.max_subs;
            it.dargs = bdargs;
            it.grid = bgrid;
            it.da = da;
            it.da.grid = bgrid;
            it.da.ik = ikmode;
            it.da.ik_dim = ikdim;
            g_batch.items.push_back(it);
            g_batch.deferred++;
            p->last_conv[1] = CONV_LINE;
            return 0;
          }
          PG_CUDA(cudaMemsetAsync(d->grid, 0, gbytes, s));
          if (fj.pending) PG_CUDA(fj.join());  // B^T needs the binning from the auxiliary stream
          {
            StageScope sc(d, PNFFT_TIMER_MATRIX_B, 1);
            if (!(cflags & PNFFT_OMIT_CONV) && nd) {
              ConvArgs c = ca;
              c.offset = off;
              c.stride = stride;
              c.f_in = fin;
              c.grad_in = gin;
              p->last_conv[1] = launch_spread(c, mode, f32, s);
            }
          }
          {
            StageScope sc(d, PNFFT_TIMER_MATRIX_F, 1);
            if (!(cflags & PNFFT_OMIT_FFT) && fft_exec(p, CUFFT_INVERSE)) return -1;
          }
          {
            StageScope sc(d, PNFFT_TIMER_MATRIX_D, 1);
            da.ik = ikmode;
            da.ik_dim = ikdim;
            if (!(cflags & PNFFT_OMIT_DECONV)) launch_deconv_crop_acc(da, f32, s);
          }
          return 0;
        };
        if (ik) {
          if ((cflags & C_F) && one(0, 0, A.f, nullptr, 0, 1, 1)) return -1;
          if (cflags & C_GRAD)
            for (int dim = 0; dim < 3; dim++)
              if (one(1, dim, A.grad, nullptr, dim, 3, 1)) return -1;
        } else {
          int mode = ((cflags & C_F) ? 1 : 0) | ((cflags & C_GRAD) ? 2 : 0);
          if (mode && one(0, 0, A.f, A.grad, 0, 1, mode)) return -1;
        }
      }
    }
    if (fj.pending) PG_CUDA(fj.join());  // every path joins the fork
    if (!p->d_f_hat_user && fb > 0) {
      if (!p->f_hat) return set_error("pnfft_adj: f_hat is not allocated"), -1;
      PG_CUDA(cudaMemcpyAsync(p->f_hat, A.fhat, fb, cudaMemcpyDeviceToHost, s));
    }
  }
  p->timer_adj[PNFFT_TIMER_ITER] += 1;
  PG_CUDA(cudaGetLastError());
  if (!(zc || !nd) || !p->d_f_hat_user) {
    PG_CUDA(cudaStreamSynchronize(s));
    engine_flush_timers(p);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// autotuning: the kernel family of each direction and the sub-problem size of
// line binnings, timed on the caller's nodes
//
// Candidates: interpolation with the line kernels (method 0) or one warp per
// node over 8x8x8 tiles (method 2, FP32-mixed); spreading with the rotating
// register window (0) or the window that moves by copies (2); line
// sub-problems of 256, 512 or 2048 nodes.  Each candidate runs `reps` timed
// calls (after one untimed call) with the node set treated as changing (it is
// binned in every call, as pnfft_trafo / pnfft_adj do), and the time of a call
// is its binning plus its convolution (stage timers).  The plan keeps, per
// direction, the fastest method, and the sub-problem size with the smallest
// sum over both directions.  The transforms write their outputs as usual.
// ---------------------------------------------------------------------------
static int time_call(pnfft_plan p, pnfft_nodes nd, bool adjoint, unsigned flags, int reps, double *ms) {
  double best = 1e300;
  for (int r = 0; r <= reps; r++) {
    nd->version++;  // re-bin as for changing coordinates
    if ((adjoint ? engine_adj(p, nd, flags) : engine_trafo(p, nd, flags)) || engine_sync(p)) return -1;
    const double t = p->last_ms[adjoint ? 1 : 0][PNFFT_TIMER_SORT_NODES] + p->last_ms[adjoint ? 1 : 0][PNFFT_TIMER_MATRIX_B];
    if (r > 0) best = std::min(best, t);
  }
  *ms = best;
  return 0;
}

int engine_autotune(pnfft_plan p, pnfft_nodes nd, unsigned trafo_flags, unsigned adj_flags, int reps) {
  if (g_batch.active)  // its calls would be deferred, not timed
    return set_error("pnfft_gb300_autotune: a batch is open (pnfft_gb300_batch_begin)"), -1;
  const int keep[2] = {p->conv_method[0], p->conv_method[1]}, keep_sub = p->line_sub_max;
  const int subs[3] = {256, 512, 2048};
  const int methods[2] = {0, 2};
  const int nm = fp32(p) ? 2 : 1;  // FP64 plans have one family per direction
  double best_total = 1e300;
  int best[3] = {keep[0], keep[1], keep_sub};
  const int fixed = nd->fixed;
  nd->fixed = 0;
  for (int si = 0; si < 3; si++) {
    p->line_sub_max = subs[si];
    double bt[2] = {1e300, 1e300};
    int bm[2] = {0, 0};
    for (int dir = 0; dir < 2; dir++) {
      const unsigned flags = dir ? adj_flags : trafo_flags;
      if (!flags) {
        bt[dir] = 0.0;
        bm[dir] = keep[dir];
        continue;
      }
      for (int mi = 0; mi < nm; mi++) {
        p->conv_method[dir] = methods[mi];
        double ms = 0.0;
        if (time_call(p, nd, dir == 1, flags, reps, &ms)) {
          p->conv_method[0] = keep[0];
          p->conv_method[1] = keep[1];
          p->line_sub_max = keep_sub;
          nd->fixed = fixed;
          return -1;
        }
        if (ms < bt[dir]) {
          bt[dir] = ms;
          bm[dir] = methods[mi];
        }
      }
      p->conv_method[dir] = bm[dir];
    }
    if (bt[0] + bt[1] < best_total) {
      best_total = bt[0] + bt[1];
      best[0] = bm[0];
      best[1] = bm[1];
      best[2] = subs[si];
    }
  }
  p->conv_method[0] = best[0];
  p->conv_method[1] = best[1];
  p->line_sub_max = best[2];
  nd->fixed = fixed;
  nd->version++;
  return 0;
}

// ---------------------------------------------------------------------------
// the charge/dipole sequence of a particle-mesh code in one call
// (tests/check_charge_dipole.c:151-233 of the reference):
//   f_hat = adj(charges, F) + adj(dipoles, GRAD_F);
//   trafo(charges, F | GRAD_F);  trafo(dipoles, GRAD_F | HESSIAN_F)
// with host arrays.  Both node sets are held fixed for the call (after one
// version bump, so that their coordinates are read once more): each is
// uploaded and binned once, and its binning serves its adjoint and its trafo
// (both directions use the line binning).  f_hat stays on the device between
// the transforms and is copied to the plan's f_hat at the end.
// ---------------------------------------------------------------------------
// energy and force of each particle: charges q phi and q grad phi, dipoles
// mu . grad phi and H mu (H in the order xx, xy, xz, yy, yz, zz)
__global__ void k_charge_dipole_results(int64_t Mc, int64_t Md, const double2 *__restrict__ q,
                                        const double2 *__restrict__ phi, const double2 *__restrict__ gc,
                                        const double2 *__restrict__ mu, const double2 *__restrict__ gd,
                                        const double2 *__restrict__ h, double2 *__restrict__ energy,
                                        double2 *__restrict__ force) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  auto mul = [](double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
  auto add = [](double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); };
  if (j < Mc) {
    energy[j] = mul(q[j], phi[j]);
    for (int t = 0; t < 3; t++) force[3 * j + t] = mul(gc[3 * j + t], q[j]);
  } else if (j < Mc + Md) {
    const int64_t k = j - Mc;
    const double2 *m = mu + 3 * k, *g = gd + 3 * k, *H = h + 6 * k;
    energy[j] = add(add(mul(g[0], m[0]), mul(g[1], m[1])), mul(g[2], m[2]));
    double2 *o = force + 3 * j;
    o[0] = add(add(mul(H[0], m[0]), mul(H[1], m[1])), mul(H[2], m[2]));
    o[1] = add(add(mul(H[1], m[0]), mul(H[3], m[1])), mul(H[4], m[2]));
    o[2] = add(add(mul(H[2], m[0]), mul(H[4], m[1])), mul(H[5], m[2]));
  }
}

int engine_charge_dipole(pnfft_plan p, pnfft_nodes ch, pnfft_nodes di, unsigned cflags, void *energy, void *force) {
  if (ensure_dev(p)) return -1;
  if (ch->u_x || di->u_x) {
    set_error("pnfft_gb300_charge_dipole: the nodes carry device arrays; this call takes host arrays");
    return -1;
  }
  if (p->d_f_hat_user) {
    set_error("pnfft_gb300_charge_dipole: the plan carries a device f_hat; this call takes the host f_hat");
    return -1;
  }
  DevState *d = p->dev;
  cudaStream_t s = d->stream;
  const int64_t Mc = ch->local_M, Md = di->local_M;
  const size_t fb = sizeof(double) * 2 * (size_t)p->local_N_total;
  if (d->fhat_cap < fb) {
    if (d->fhat) cudaFree(d->fhat);
    d->fhat = nullptr;
    d->fhat_cap = 0;
    PG_CUDA(cudaMalloc(&d->fhat, fb > 0 ? fb : 16));
    d->fhat_cap = fb;
  }
  // q (Mc), mu (3 Md), energy (Mc + Md), force (3 (Mc + Md)) on the device
  double2 *buf = nullptr;
  const size_t nbuf = (size_t)(Mc + 3 * Md + 4 * (Mc + Md));
  PG_CUDA(cudaMallocAsync(&buf, sizeof(double2) * std::max<size_t>(nbuf, 1), s));
  double2 *q = buf, *mu = q + Mc, *en = mu + 3 * Md, *fo = en + (Mc + Md);
  const int fixed_ch = ch->fixed, fixed_di = di->fixed;
  ch->version++;
  di->version++;
  ch->fixed = di->fixed = 1;
  p->d_f_hat_user = d->fhat;
  const unsigned extra = cflags & ~(PNFFT_COMPUTE_F | PNFFT_COMPUTE_GRAD_F | PNFFT_COMPUTE_HESSIAN_F |
                                    PNFFT_COMPUTE_ACCUMULATED);
  auto keep = [&](double2 *dst, const double *src, int64_t count) -> int {  // device copy of an input
    if (count > 0 && cudaMemcpyAsync(dst, src, sizeof(double2) * count, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      set_error("pnfft_gb300_charge_dipole: keeping the inputs failed");
      return -1;
    }
    return 0;
  };
  int rc = engine_adj(p, ch, extra | PNFFT_COMPUTE_F);
  if (!rc && Mc > 0) rc = keep(q, ch->dev->f, Mc);  // uploaded by the adjoint
  if (!rc) rc = engine_adj(p, di, extra | PNFFT_COMPUTE_GRAD_F | PNFFT_COMPUTE_ACCUMULATED);
  if (!rc && Md > 0) rc = keep(mu, di->dev->grad, 3 * Md);
  if (!rc) rc = engine_trafo(p, ch, extra | PNFFT_COMPUTE_F | PNFFT_COMPUTE_GRAD_F);
  if (!rc) rc = engine_trafo(p, di, extra | PNFFT_COMPUTE_GRAD_F | PNFFT_COMPUTE_HESSIAN_F);
  p->d_f_hat_user = nullptr;
  ch->fixed = fixed_ch;
  di->fixed = fixed_di;
  if (!rc && (energy || force) && Mc + Md > 0) {
    const double2 *none = nullptr;
    k_charge_dipole_results<<<(unsigned)((Mc + Md + 255) / 256), 256, 0, s>>>(
        Mc, Md, q, Mc ? (const double2 *)ch->dev->f : none, Mc ? (const double2 *)ch->dev->grad : none, mu,
        Md ? (const double2 *)di->dev->grad : none, Md ? (const double2 *)di->dev->hess : none, en, fo);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && energy)
      e = cudaMemcpyAsync(energy, en, sizeof(double2) * (Mc + Md), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && force)
      e = cudaMemcpyAsync(force, fo, sizeof(double2) * 3 * (Mc + Md), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) {
      set_error("pnfft_gb300_charge_dipole: the energies and forces failed: %s", cudaGetErrorString(e));
      rc = -1;
    }
  }
  if (!rc && fb > 0 && p->f_hat) {
    cudaError_t e = cudaMemcpyAsync(p->f_hat, d->fhat, fb, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) {
      set_error("pnfft_gb300_charge_dipole: copying f_hat back failed: %s", cudaGetErrorString(e));
      rc = -1;
    }
  }
  cudaFreeAsync(buf, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (!rc && e != cudaSuccess) {
    set_error("pnfft_gb300_charge_dipole: %s", cudaGetErrorString(e));
    rc = -1;
  }
  engine_flush_timers(p);
  return rc;
}

// ---------------------------------------------------------------------------
// misc
// ---------------------------------------------------------------------------
int engine_set_stream(pnfft_plan p, void *stream) {
  p->user_stream = stream;
  if (p->dev && p->dev->device >= 0) {
    p->dev->stream = stream ? (cudaStream_t)stream : p->dev->own;
    if (p->dev->fft_prec >= 0) PG_FFT(cufftSetStream(p->dev->fft, p->dev->stream));
  }
  return 0;
}

int engine_sync(pnfft_plan p) {
  if (!p->dev || p->dev->device < 0) return 0;
  PG_CUDA(cudaStreamSynchronize(p->dev->stream));
  engine_flush_timers(p);
  return 0;
}

void engine_release_plan(pnfft_plan p) {
  DevState *d = p->dev;
  if (!d) return;
  for (const Deferred &it : g_batch.items)
    if (it.p == p) {
      batch_flush();  // the plan's deferred calls run before its buffers go
      break;
    }
  g_batch.plans.erase(std::remove(g_batch.plans.begin(), g_batch.plans.end(), p), g_batch.plans.end());
  if (d->device >= 0) {
    cudaStreamSynchronize(d->stream);
    for (void *g : d->bgrid) cudaFree(g);  // cudaFree waits for the device
    for (ConvArgs *a : d->bargs) cudaFree(a);
    for (cudaEvent_t e : d->bev) cudaEventDestroy(e);
    d->pending.clear();
    if (d->grid) cudaFree(d->grid);
    if (d->fft_prec >= 0) cufftDestroy(d->fft);
    for (int t = 0; t < 3; t++)
      if (d->inv[t]) cudaFree(d->inv[t]);
    for (int a = 0; a < 3; a++)
      for (int t = 0; t < 3; t++)
        if (d->tab[a][t]) cudaFree(d->tab[a][t]);
    if (d->fhat) cudaFree(d->fhat);
    if (d->poly) cudaFree(d->poly);
    for (cudaEvent_t e : d->free_ev) cudaEventDestroy(e);
    if (d->own) cudaStreamDestroy(d->own);
    if (d->aux) cudaStreamDestroy(d->aux);
    if (d->ev_fork) cudaEventDestroy(d->ev_fork);
    if (d->ev_join) cudaEventDestroy(d->ev_join);
    cudaGetLastError();
  }
  delete d;
  p->dev = nullptr;
}

void engine_release_nodes(pnfft_nodes nd) {
  NodeDev *v = nd->dev;
  if (!v) return;
  for (const Deferred &it : g_batch.items)
    if (it.slot == &v->bins[0][0]) {
      batch_flush();  // deferred calls read this node set's binning: they run first
      break;
    }
  cudaFree(v->x);  // cudaFree waits for the device
  cudaFree(v->f);
  cudaFree(v->grad);
  cudaFree(v->hess);
  for (auto &row : v->bins)
    for (auto &sl : row) free_binning(sl.b);
  cudaGetLastError();
  delete v;
  nd->dev = nullptr;
}

int engine_sort_nodes(pnfft_plan p, int64_t M, const double *x, long long *pairs) {
  if (ensure_dev(p)) return -1;
  cudaStream_t s = p->dev->stream;
  if (M <= 0) return 0;
  double *dx = nullptr;
  long long *dp = nullptr;
  PG_CUDA(cudaMallocAsync(&dx, sizeof(double) * 3 * M, s));
  PG_CUDA(cudaMallocAsync(&dp, sizeof(long long) * 2 * M, s));
  PG_CUDA(cudaMemcpyAsync(dx, x, sizeof(double) * 3 * M, cudaMemcpyHostToDevice, s));
  int n[3] = {(int)p->n[0], (int)p->n[1], (int)p->n[2]};
  int rc = radix_sort_nodes(dx, M, n, p->m, dp, s);
  if (rc == 0) PG_CUDA(cudaMemcpyAsync(pairs, dp, sizeof(long long) * 2 * M, cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(dx, s);
  cudaFreeAsync(dp, s);
  PG_CUDA(cudaStreamSynchronize(s));
  if (rc) set_error("pnfft_gb300_sort_nodes: device allocation failed");
  return rc;
}

int engine_node_index(pnfft_plan p, int64_t M, const double *x, int interlaced, long long *u) {
  if (ensure_dev(p)) return -1;
  cudaStream_t s = p->dev->stream;
  if (M <= 0) return 0;
  double *dx = nullptr;
  long long *du = nullptr;
  PG_CUDA(cudaMallocAsync(&dx, sizeof(double) * 3 * M, s));
  PG_CUDA(cudaMallocAsync(&du, sizeof(long long) * 3 * M, s));
  PG_CUDA(cudaMemcpyAsync(dx, x, sizeof(double) * 3 * M, cudaMemcpyHostToDevice, s));
  int n[3] = {(int)p->n[0], (int)p->n[1], (int)p->n[2]};
  launch_node_index(dx, M, n, p->m, interlaced, fp32(p), du, s);
  PG_CUDA(cudaMemcpyAsync(u, du, sizeof(long long) * 3 * M, cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(dx, s);
  cudaFreeAsync(du, s);
  PG_CUDA(cudaStreamSynchronize(s));
  return 0;
}

}  // namespace pg
