// api.cpp -- the C ABI of libpnfft_gb300: the pnfft_* entry points of
// include/pnfft.h (double precision, 1x1x1 process mesh) and the
// pnfft_gb300_* extensions of include/pnfft_gb300.h.
//
// Host-side plan logic restates the reference's: plan creation
// (api/api-guru.c:110-164, kernel/ndft-parallel.c:869-1140), window shape b,
// interpolation tables (ndft-parallel.c:321-353, 1088-1122), the window
// Fourier coefficients (kernel/matrix_D.c:30-225), getters/setters
// (api/api-basic.c:457-661), node objects (380-447), timers
// (kernel/timer.c) and the command-line helpers (api-basic.c:820-953).
// All numerical work of pnfft_trafo / pnfft_adj runs on the GPU (engine.cu).
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <string>

#include "pg_internal.h"
#include "pg_math.cuh"

using pg::set_error;

namespace pg {

static thread_local std::string g_err;

void set_error(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}
const char *last_error() { return g_err.c_str(); }

static std::atomic<uint64_t> g_uid{1};

// Re erf(a + i y) = erf(a) + 2/sqrt(pi) e^{-a^2} int_0^y e^{t^2} sin(2 a t) dt,
// integral by Romberg extrapolation of the trapezoidal rule.
static double re_erf_complex(double a, double y) {
  if (y == 0.0) return erf(a);
  auto g = [a](double t) { return exp(t * t - a * a) * sin(2.0 * a * t); };
  const int K = 18;
  double R[K][K];
  double h = y;
  R[0][0] = 0.5 * h * (g(0.0) + g(y));
  int used = 1;
  for (int i = 1; i < K; i++) {
    h *= 0.5;
    double s = 0;
    long long np = 1LL << (i - 1);
    for (long long k = 0; k < np; k++) s += g((2 * k + 1) * h);
    R[i][0] = 0.5 * R[i - 1][0] + h * s;
    double p4 = 4.0;
    for (int j = 1; j <= i; j++) {
      R[i][j] = R[i][j - 1] + (R[i][j - 1] - R[i - 1][j - 1]) / (p4 - 1.0);
      p4 *= 4.0;
    }
    used = i + 1;
    if (i > 4 && fabs(R[i][i] - R[i - 1][i - 1]) <= 1e-16 * fabs(R[i][i]) + 1e-300) break;
  }
  return erf(a) + 2.0 / sqrt(kPi) * R[used - 1][used - 1];
}

// window Fourier coefficient of axis t at frequency k, kernel/matrix_D.c:209-225
static double phi_hat_host(const pnfft_plan p, int t, int64_t k) {
  const double n = (double)p->n[t], b = p->b[t];
  const int m = p->m;
  switch (p->window) {
    case WIN_GAUSSIAN: {
      double q = kPi * (double)k / n;
      if (p->gauss_t) {
        double sb = sqrt(b);
        return exp(-q * q * b) * re_erf_complex((double)m / sb, kPi * (double)k * sb / n);
      }
      return exp(-q * q * b);
    }
    case WIN_BSPLINE:
      return pow(sinc<double>((double)k * kPi / n), 2.0 * m);
    case WIN_SINC_POWER:
      return bspline<double>(2 * m, fabs((double)k * b / n) + m);
    case WIN_BESSEL_I0: {
      double q = 2.0 * kPi * (double)k / n, d = b * b - q * q;
      double r = (d < 0) ? sqrt(-d) : sqrt(d);
      if (d < 0) return sin(m * r) / r;
      return (d > 0) ? sinh(m * r) / r : (double)m;
    }
    default: {
      double q = 2.0 * kPi * (double)k / n, d = b * b - q * q;
      if (d < 0) return 0.0;
      return (d > 0) ? bessel_i0<double>(m * sqrt(d)) : 1.0;
    }
  }
}

// inverse coefficient, matrix_D.c:191-207 (zero where the reference returns 0)
static double inv_phi_hat_host(const pnfft_plan p, int t, int64_t k) {
  const double n = (double)p->n[t], b = p->b[t];
  const int m = p->m;
  switch (p->window) {
    case WIN_GAUSSIAN: {
      if (p->gauss_t) return 1.0 / phi_hat_host(p, t, k);
      double q = kPi * (double)k / n;
      return exp(q * q * b);
    }
    case WIN_BSPLINE:
      return pow(sinc<double>((double)k * kPi / n), -2.0 * m);
    case WIN_SINC_POWER: {
      double d = fabs((double)k * b / n);
      return (d < m) ? 1.0 / bspline<double>(2 * m, d + m) : 0.0;
    }
    case WIN_BESSEL_I0: {
      double q = 2.0 * kPi * (double)k / n, d = b * b - q * q;
      double r = (d < 0) ? sqrt(-d) : sqrt(d);
      if (d < 0) return r / sin(m * r);
      return (d > 0) ? r / sinh(m * r) : 1.0 / m;
    }
    default: {
      double q = 2.0 * kPi * (double)k / n, d = b * b - q * q;
      if (d < 0) return 0.0;
      return (d > 0) ? 1.0 / bessel_i0<double>(m * sqrt(d)) : 1.0;
    }
  }
}

static double window_host(const pnfft_plan p, int t, double x, int der) {
  return window_1d<double>(p->window, p->m, (double)p->n[t], p->b[t], x, der);
}

// deconvolution factors and interpolation tables; called at creation and by set_b
static void init_precompute_window(pnfft_plan p) {
  for (int t = 0; t < 3; t++) {
    p->inv[t].resize((size_t)p->local_N[t]);
    for (int64_t k = 0; k < p->local_N[t]; k++) p->inv[t][k] = inv_phi_hat_host(p, t, p->local_N_start[t] + k);
  }
  for (int der = 0; der < 3; der++)
    for (int t = 0; t < 3; t++) p->tab[der][t].clear();
  if (p->intpol_order >= 0) {
    const int ord = p->intpol_order, cut = p->cutoff;
    const int64_t K = (int64_t)ceil((2.0 * 15.0 + 1.0) / cut) * 2048;  // ndft-parallel.c:1095
    p->intpol_K = K;
    const int nder = (p->pnfft_flags & PNFFT_DIFF_IK) ? 1 : 3;  // 1105
    for (int der = 0; der < nder; der++)
      for (int t = 0; t < 3; t++) {
        std::vector<double> &tab = p->tab[der][t];
        tab.resize((size_t)K * cut * (ord + 1));
        size_t ind = 0;
        for (int64_t k = 0; k < K; k++)
          for (int c = 0; c < cut; c++)
            for (int i = -ord / 2; i <= (ord + 1) / 2; i++, ind++)
              tab[ind] = window_host(p, t, (p->m + (double)(k + i) / (double)K - c) / (double)p->n[t], der);
      }
  }
  p->table_version++;
}

}  // namespace pg

using namespace pg;

// ===========================================================================
// process mesh, local sizes
// ===========================================================================
extern "C" int pnfft_create_procmesh_2d(MPI_Comm comm, int np0, int np1, MPI_Comm *comm_cart_2d) {
  if ((long long)np0 * np1 != 1) {
    set_error("pnfft_create_procmesh_2d: libpnfft_gb300 runs one process per GPU (1 x 1 mesh only)");
    return 1;
  }
  if (comm_cart_2d) *comm_cart_2d = comm;
  return 0;
}

extern "C" int pnfft_create_procmesh(int rnk, MPI_Comm comm, const int *np, MPI_Comm *comm_cart) {
  long long tot = 1;
  for (int t = 0; t < rnk; t++) tot *= np[t];
  if (tot != 1) {
    set_error("pnfft_create_procmesh: libpnfft_gb300 runs one process per GPU (1 x 1 x 1 mesh only)");
    return 1;
  }
  if (comm_cart) *comm_cart = comm;
  return 0;
}

// no = min(n, 2 (floor(n x_max) + m + 2)), api/api-guru.c:195-218
static void fft_output_size(const ptrdiff_t *n, const double *x_max, int m, int64_t *no) {
  for (int t = 0; t < 3; t++) {
    int64_t c = (int64_t)lrint(floor((double)n[t] * x_max[t]));
    int64_t v = 2 * (c + m + 2);
    no[t] = n[t] < v ? n[t] : v;
  }
}

static void local_size_internal(int c2r, const ptrdiff_t *N, const ptrdiff_t *n, const double *x_max, int m,
                                ptrdiff_t *local_N, ptrdiff_t *local_N_start, double *lo, double *up) {
  int64_t no[3];
  fft_output_size(n, x_max, m, no);
  for (int t = 0; t < 3; t++) {
    local_N[t] = N[t];
    local_N_start[t] = -(N[t] / 2);
  }
  if (c2r) local_N[2] = N[2] / 2 + 1;  // half spectrum k2 in [-N2/2, 0]
  for (int t = 0; t < 3; t++) {        // node_borders, ndft-parallel.c:734-775
    double l = (double)(-(no[t] / 2)) / (double)n[t];
    double u = (double)(-(no[t] / 2) + no[t]) / (double)n[t];
    if (l < -x_max[t]) l = -x_max[t];
    if (l > x_max[t]) l = x_max[t];
    if (u < -x_max[t]) u = -x_max[t];
    if (u > x_max[t]) u = x_max[t];
    if (lo) lo[t] = l;
    if (up) up[t] = u;
  }
}

extern "C" void pnfft_local_size_guru(int d, const ptrdiff_t *N, const ptrdiff_t *n, const double *x_max, int m,
                                      MPI_Comm, unsigned, ptrdiff_t *local_N, ptrdiff_t *local_N_start,
                                      double *lower_border, double *upper_border) {
  if (d != 3) {
    set_error("!!! Error in PNFFT: d != 3 not yet implemented !!!");
    fprintf(stderr, "!!! Error in PNFFT: d != 3 not yet implemented !!!\n");
    return;
  }
  local_size_internal(0, N, n, x_max, m, local_N, local_N_start, lower_border, upper_border);
}

extern "C" void pnfft_local_size_guru_c2r(int d, const ptrdiff_t *N, const ptrdiff_t *n, const double *x_max, int m,
                                          MPI_Comm, unsigned, ptrdiff_t *local_N, ptrdiff_t *local_N_start,
                                          double *lower_border, double *upper_border) {
  if (d != 3) {
    set_error("!!! Error in PNFFT: d != 3 not yet implemented !!!");
    fprintf(stderr, "!!! Error in PNFFT: d != 3 not yet implemented !!!\n");
    return;
  }
  local_size_internal(1, N, n, x_max, m, local_N, local_N_start, lower_border, upper_border);
}

// defaults of api/api-adv.c:172-192: n = 2N, x_max = 0.5, m = 6
static void adv_defaults(const ptrdiff_t *N, ptrdiff_t *n, double *x_max, int *m) {
  for (int t = 0; t < 3; t++) {
    n[t] = 2 * N[t];
    x_max[t] = 0.5;
  }
  *m = 6;
}

extern "C" void pnfft_local_size_adv(int d, const ptrdiff_t *N, MPI_Comm comm, unsigned flags, ptrdiff_t *local_N,
                                     ptrdiff_t *local_N_start, double *lo, double *up) {
  ptrdiff_t n[3];
  double xm[3];
  int m;
  adv_defaults(N, n, xm, &m);
  pnfft_local_size_guru(d, N, n, xm, m, comm, flags, local_N, local_N_start, lo, up);
}

extern "C" void pnfft_local_size_adv_c2r(int d, const ptrdiff_t *N, MPI_Comm comm, unsigned flags,
                                         ptrdiff_t *local_N, ptrdiff_t *local_N_start, double *lo, double *up) {
  ptrdiff_t n[3];
  double xm[3];
  int m;
  adv_defaults(N, n, xm, &m);
  pnfft_local_size_guru_c2r(d, N, n, xm, m, comm, flags, local_N, local_N_start, lo, up);
}

extern "C" void pnfft_local_size_3d(const ptrdiff_t *N, MPI_Comm comm, unsigned flags, ptrdiff_t *local_N,
                                    ptrdiff_t *local_N_start, double *lo, double *up) {
  pnfft_local_size_adv(3, N, comm, flags, local_N, local_N_start, lo, up);
}

extern "C" void pnfft_local_size_3d_c2r(const ptrdiff_t *N, MPI_Comm comm, unsigned flags, ptrdiff_t *local_N,
                                        ptrdiff_t *local_N_start, double *lo, double *up) {
  pnfft_local_size_adv_c2r(3, N, comm, flags, local_N, local_N_start, lo, up);
}

// ===========================================================================
// plans
// ===========================================================================
static unsigned extract_pfft_opt_flags(unsigned f) {  // api/api-guru.c:168-190
  unsigned r = 0;
  if (f & PFFT_ESTIMATE) r = PFFT_ESTIMATE;
  if (f & PFFT_PATIENT) r = PFFT_PATIENT;
  if (f & PFFT_EXHAUSTIVE) r = PFFT_EXHAUSTIVE;
  if (f & PFFT_TUNE) r |= PFFT_TUNE;
  if (f & PFFT_PRESERVE_INPUT) r |= PFFT_PRESERVE_INPUT;
  if (f & PFFT_DESTROY_INPUT) r |= PFFT_DESTROY_INPUT;
  return r;
}

// The radial windows grow like exp(b m): Kaiser-Bessel and Bessel-I0 with
// b m >= 80 (m >= 17 at oversampling 2) overflow FP32, so FP32-mixed plans
// refuse them.
static bool fp32_window_in_range(const pnfft_plan p) {
  if (p->window != WIN_KAISER_BESSEL && p->window != WIN_BESSEL_I0) return true;
  for (int t = 0; t < 3; t++)
    if (p->b[t] * (double)p->m >= 80.0) {
      set_error("FP32-mixed precision: the %s window with m=%d overflows FP32 (b*m=%.1f >= 80); use FP64",
                p->window == WIN_KAISER_BESSEL ? "Kaiser-Bessel" : "Bessel-I0", p->m, p->b[t] * (double)p->m);
      return false;
    }
  return true;
}

static pnfft_plan init_guru_internal(int d, const ptrdiff_t *N, const ptrdiff_t *n, const double *x_max, int m,
                                     int c2r, unsigned pnfft_flags, unsigned pfft_flags) {
  if (d != 3) {
    set_error("!!! Error in PNFFT: d != 3 not yet implemented !!!");
    fprintf(stderr, "!!! Error in PNFFT: d != 3 not yet implemented !!!\n");
    return NULL;
  }
  for (int t = 0; t < 3; t++) {
    if (N[t] < 1 || n[t] < N[t] || n[t] > (1 << 20)) {
      set_error("pnfft_init: invalid sizes N[%d]=%td n[%d]=%td (need 1 <= N <= n)", t, N[t], t, n[t]);
      return NULL;
    }
  }
  if (m < 1 || 2 * m + 1 > 63) {
    set_error("pnfft_init: cutoff m=%d outside [1, 31]", m);
    return NULL;
  }
  // flag promotion, api/api-guru.c:152-155 (precompute-flag values tested on
  // plan flags: PNFFT_PRE_HESSIAN_PSI == PRE_LIN_PSI, PRE_GRAD_PSI == PRE_CONST_PSI)
  if (pnfft_flags & PNFFT_PRE_HESSIAN_PSI) pnfft_flags |= PNFFT_PRE_GRAD_PSI;
  if (pnfft_flags & PNFFT_PRE_GRAD_PSI) pnfft_flags |= PNFFT_PRE_PSI;

  pnfft_plan p = new pnfft_plan_s();
  p->line_sub_max = 512;
  p->d = 3;
  p->m = m;
  p->cutoff = 2 * m + 1;
  p->c2r = c2r;
  p->pnfft_flags = pnfft_flags;
  p->pfft_flags = extract_pfft_opt_flags(pfft_flags);
  for (int t = 0; t < 3; t++) {
    p->N[t] = N[t];
    p->n[t] = n[t];
    p->x_max[t] = x_max[t];
    p->sigma[t] = (double)n[t] / (double)N[t];
  }
  fft_output_size(n, x_max, m, p->no);
  ptrdiff_t lN[3], lNs[3];
  local_size_internal(c2r, N, n, x_max, m, lN, lNs, NULL, NULL);
  p->local_N_total = 1;
  for (int t = 0; t < 3; t++) {
    p->local_N[t] = lN[t];
    p->local_N_start[t] = lNs[t];
    p->local_N_total *= lN[t];
    p->local_no[t] = p->no[t];
    p->local_no_start[t] = -(p->no[t] / 2);
  }
  if (pnfft_flags & PNFFT_WINDOW_GAUSSIAN) p->window = WIN_GAUSSIAN;
  else if (pnfft_flags & PNFFT_WINDOW_BSPLINE) p->window = WIN_BSPLINE;
  else if (pnfft_flags & PNFFT_WINDOW_SINC_POWER) p->window = WIN_SINC_POWER;
  else if (pnfft_flags & PNFFT_WINDOW_BESSEL_I0) p->window = WIN_BESSEL_I0;
  else p->window = WIN_KAISER_BESSEL;
  p->gauss_t = (p->window == WIN_GAUSSIAN) && (pnfft_flags & PNFFT_USE_FK_GAUSSIAN_T);
  // interpolation order, ndft-parallel.c:997-1006
  if (pnfft_flags & PNFFT_PRE_CONST_PSI) p->intpol_order = 0;
  else if (pnfft_flags & PNFFT_PRE_LIN_PSI) p->intpol_order = 1;
  else if (pnfft_flags & PNFFT_PRE_QUAD_PSI) p->intpol_order = 2;
  else if (pnfft_flags & PNFFT_PRE_CUB_PSI) p->intpol_order = 3;
  else p->intpol_order = -1;
  // window shape, ndft-parallel.c:1008-1064
  for (int t = 0; t < 3; t++) {
    double s = p->sigma[t];
    switch (p->window) {
      case WIN_GAUSSIAN: p->b[t] = ((double)m / kPi) * 2.0 * s / (2.0 * s - 1.0); break;
      case WIN_BSPLINE: p->b[t] = 0.0; break;
      case WIN_SINC_POWER: p->b[t] = (double)m * (2.0 * s) / (2.0 * s - 1.0); break;
      default: p->b[t] = kPi * (2.0 - 1.0 / s); break;
    }
  }
  p->precision = (pnfft_flags & PNFFT_GB300_FP32) ? PNFFT_GB300_FP32_MIXED : PNFFT_GB300_FP64;
  if (p->precision == PNFFT_GB300_FP32_MIXED && !fp32_window_in_range(p)) {
    delete p;
    return nullptr;
  }
  p->uid = g_uid.fetch_add(1);
  if (pnfft_flags & PNFFT_MALLOC_F_HAT) {
    p->f_hat = pnfft_malloc(sizeof(double) * 2 * (size_t)p->local_N_total);
    p->own_f_hat = 1;
    if (p->f_hat) memset(p->f_hat, 0, sizeof(double) * 2 * (size_t)p->local_N_total);
  }
  init_precompute_window(p);
  return p;
}

extern "C" pnfft_plan pnfft_init_guru(int d, const ptrdiff_t *N, const ptrdiff_t *n, const double *x_max, int m,
                                      unsigned pnfft_flags, unsigned pfft_flags, MPI_Comm) {
  return init_guru_internal(d, N, n, x_max, m, 0, pnfft_flags, pfft_flags);
}

extern "C" pnfft_plan pnfft_init_guru_c2r(int d, const ptrdiff_t *N, const ptrdiff_t *n, const double *x_max, int m,
                                          unsigned pnfft_flags, unsigned pfft_flags, MPI_Comm) {
  return init_guru_internal(d, N, n, x_max, m, 1, pnfft_flags, pfft_flags);
}

extern "C" pnfft_plan pnfft_init_adv(int d, const ptrdiff_t *N, unsigned pnfft_flags, unsigned pfft_flags,
                                     MPI_Comm comm) {
  ptrdiff_t n[3];
  double xm[3];
  int m;
  adv_defaults(N, n, xm, &m);
  return pnfft_init_guru(d, N, n, xm, m, pnfft_flags, pfft_flags, comm);
}

extern "C" pnfft_plan pnfft_init_adv_c2r(int d, const ptrdiff_t *N, unsigned pnfft_flags, unsigned pfft_flags,
                                         MPI_Comm comm) {
  ptrdiff_t n[3];
  double xm[3];
  int m;
  adv_defaults(N, n, xm, &m);
  return pnfft_init_guru_c2r(d, N, n, xm, m, pnfft_flags, pfft_flags, comm);
}

extern "C" pnfft_plan pnfft_init_3d(const ptrdiff_t *N, MPI_Comm comm) {
  return pnfft_init_adv(3, N, PNFFT_MALLOC_F_HAT, PFFT_MEASURE | PFFT_DESTROY_INPUT, comm);
}

extern "C" pnfft_plan pnfft_init_3d_c2r(const ptrdiff_t *N, MPI_Comm comm) {
  return pnfft_init_adv_c2r(3, N, PNFFT_MALLOC_F_HAT, PFFT_MEASURE | PFFT_DESTROY_INPUT, comm);
}

extern "C" void pnfft_finalize(pnfft_plan ths, unsigned flags) {
  if (!ths) return;
  engine_release_plan(ths);
  if ((flags & PNFFT_FREE_F_HAT) && ths->f_hat) pnfft_free(ths->f_hat);
  delete ths;
}

// ===========================================================================
// nodes
// ===========================================================================
extern "C" pnfft_nodes pnfft_init_nodes(ptrdiff_t local_M, unsigned malloc_flags) {
  if (local_M < 0) {
    set_error("pnfft_init_nodes: local_M < 0");
    return NULL;
  }
  pnfft_nodes nd = new pnfft_nodes_s();
  nd->local_M = local_M;
  nd->uid = g_uid.fetch_add(1);
  nd->version = 1;
  size_t M = (size_t)local_M;
  if (M > 0) {  // api-basic.c:412-415, ndft-parallel.c:1484-1522
    if (malloc_flags & PNFFT_MALLOC_X) nd->x = pnfft_alloc_real(3 * M);
    if (malloc_flags & PNFFT_MALLOC_F) nd->f = pnfft_alloc_real(2 * M);
    if (malloc_flags & PNFFT_MALLOC_GRAD_F) nd->grad_f = pnfft_alloc_real(6 * M);
    if (malloc_flags & PNFFT_MALLOC_HESSIAN_F) nd->hessian_f = pnfft_alloc_real(12 * M);
  }
  return nd;
}

extern "C" void pnfft_free_nodes(pnfft_nodes nd, unsigned flags) {
  if (!nd) return;
  engine_release_nodes(nd);
  if (flags & PNFFT_FREE_GRAD_F) pnfft_free(nd->grad_f);
  if (flags & PNFFT_FREE_HESSIAN_F) pnfft_free(nd->hessian_f);
  if (flags & PNFFT_FREE_F) pnfft_free(nd->f);
  if (flags & PNFFT_FREE_X) pnfft_free(nd->x);
  delete nd;
}

// The window values of the nodes are evaluated on the fly on the GPU (they are
// the same numbers the reference stores, ndft-parallel.c:1144-1370); what the
// call keeps is its promise that the coordinates stay fixed, so the node
// binning is computed once and reused.
extern "C" void pnfft_precompute_psi(pnfft_plan ths, pnfft_nodes nodes, unsigned precompute_flags) {
  (void)ths;
  if (!nodes) return;
  nodes->precompute_flags = precompute_flags;
  nodes->fixed = (precompute_flags & PNFFT_PRE_PSI) ? 1 : 0;
  nodes->version++;
}

// ===========================================================================
// setters / getters (api-basic.c:457-661)
// ===========================================================================
extern "C" void pnfft_set_f_hat(pnfft_complex *f_hat, pnfft_plan ths) { ths->f_hat = (void *)f_hat; }
extern "C" pnfft_complex *pnfft_get_f_hat(const pnfft_plan ths) { return (pnfft_complex *)ths->f_hat; }
extern "C" void pnfft_set_f_hat_real(double *f_hat, pnfft_plan ths) { ths->f_hat = f_hat; }
extern "C" double *pnfft_get_f_hat_real(const pnfft_plan ths) { return (double *)ths->f_hat; }
extern "C" void pnfft_set_f(pnfft_complex *f, pnfft_nodes nodes) { nodes->f = (double *)f; }
extern "C" pnfft_complex *pnfft_get_f(const pnfft_nodes nodes) { return (pnfft_complex *)nodes->f; }
extern "C" void pnfft_set_grad_f(pnfft_complex *g, pnfft_nodes nodes) { nodes->grad_f = (double *)g; }
extern "C" pnfft_complex *pnfft_get_grad_f(const pnfft_nodes nodes) { return (pnfft_complex *)nodes->grad_f; }
extern "C" void pnfft_set_hessian_f(pnfft_complex *h, pnfft_nodes nodes) { nodes->hessian_f = (double *)h; }
extern "C" pnfft_complex *pnfft_get_hessian_f(const pnfft_nodes nodes) { return (pnfft_complex *)nodes->hessian_f; }
extern "C" void pnfft_set_f_real(double *f, pnfft_nodes nodes) { nodes->f = f; }
extern "C" double *pnfft_get_f_real(const pnfft_nodes nodes) { return nodes->f; }
extern "C" void pnfft_set_grad_f_real(double *g, pnfft_nodes nodes) { nodes->grad_f = g; }
extern "C" double *pnfft_get_grad_f_real(const pnfft_nodes nodes) { return nodes->grad_f; }
extern "C" void pnfft_set_hessian_f_real(double *h, pnfft_nodes nodes) { nodes->hessian_f = h; }
extern "C" double *pnfft_get_hessian_f_real(const pnfft_nodes nodes) { return nodes->hessian_f; }
extern "C" void pnfft_set_x(double *x, pnfft_nodes nodes) {
  if (nodes->x != x) nodes->version++;
  nodes->x = x;
}
extern "C" double *pnfft_get_x(const pnfft_nodes nodes) { return nodes->x; }

extern "C" void pnfft_set_b(double b0, double b1, double b2, pnfft_plan ths) {
  ths->b[0] = b0;
  ths->b[1] = b1;
  ths->b[2] = b2;
  init_precompute_window(ths);
}
extern "C" void pnfft_get_b(const pnfft_plan ths, double *b0, double *b1, double *b2) {
  *b0 = ths->b[0];
  *b1 = ths->b[1];
  *b2 = ths->b[2];
}
extern "C" int pnfft_get_d(const pnfft_plan ths) { return ths->d; }
extern "C" int pnfft_get_m(const pnfft_plan ths) { return ths->m; }
extern "C" void pnfft_get_x_max(const pnfft_plan ths, double *x_max) {
  for (int t = 0; t < 3; t++) x_max[t] = ths->x_max[t];
}
extern "C" void pnfft_get_N(const pnfft_plan ths, ptrdiff_t *N) {
  for (int t = 0; t < 3; t++) N[t] = ths->N[t];
}
extern "C" void pnfft_get_n(const pnfft_plan ths, ptrdiff_t *n) {
  for (int t = 0; t < 3; t++) n[t] = ths->n[t];
}
extern "C" unsigned pnfft_get_pnfft_flags(const pnfft_plan ths) { return ths->pnfft_flags; }
extern "C" unsigned pnfft_get_pfft_flags(const pnfft_plan ths) { return ths->pfft_flags; }

// ===========================================================================
// transforms
// ===========================================================================
extern "C" void pnfft_trafo(pnfft_plan ths, pnfft_nodes nodes, unsigned compute_flags) {
  if (ths == NULL) return;  // api-basic.c:205-206
  if (nodes == NULL && (~compute_flags & PNFFT_OMIT_CONV)) return;
  if (engine_trafo(ths, nodes, compute_flags)) fprintf(stderr, "pnfft_trafo: %s\n", last_error());
}

extern "C" void pnfft_adj(pnfft_plan ths, pnfft_nodes nodes, unsigned compute_flags) {
  if (ths == NULL) return;  // api-basic.c:350-351
  if (nodes == NULL && (~compute_flags & PNFFT_OMIT_CONV)) return;
  if (engine_adj(ths, nodes, compute_flags)) fprintf(stderr, "pnfft_adj: %s\n", last_error());
}

// The charge/dipole sequence of a particle-mesh code in one call, with the
// per-particle energies and forces that the reference's particle test forms
// after it (tests/check_charge_dipole.c:151-233): charges q = charges->f at
// charges->x, dipole moments mu = dipoles->grad_f at dipoles->x.  On return
// the node arrays hold what the four reference calls leave there (charges: f =
// phi, grad_f = grad phi; dipoles: grad_f = grad phi, hessian_f = H), the plan's
// f_hat holds the spectrum, and energy / force (Mc + Md and 3 (Mc + Md)
// complex, may be NULL) hold q phi, q grad phi, mu . grad phi and H mu.
extern "C" int pnfft_gb300_charge_dipole(pnfft_plan ths, pnfft_nodes charges, pnfft_nodes dipoles,
                                         unsigned compute_flags, void *energy, void *force) {
  if (!ths || !charges || !dipoles) {
    set_error("pnfft_gb300_charge_dipole: plan and both node sets are required");
    return -1;
  }
  if (ths->c2r) {
    set_error("pnfft_gb300_charge_dipole: the sequence takes complex node values (a c2c plan)");
    return -1;
  }
  const int64_t Mc = charges->local_M, Md = dipoles->local_M;
  if ((Mc > 0 && (!charges->x || !charges->f || !charges->grad_f)) ||
      (Md > 0 && (!dipoles->x || !dipoles->grad_f || !dipoles->hessian_f))) {
    set_error("pnfft_gb300_charge_dipole: charges need x, f and grad_f; dipoles need x, grad_f and hessian_f");
    return -1;
  }
  return engine_charge_dipole(ths, charges, dipoles, compute_flags, energy, force);
}

extern "C" void pnfft_zero_f_hat(pnfft_plan ths) {  // api-basic.c:335-341
  if (ths && ths->f_hat) memset(ths->f_hat, 0, sizeof(double) * 2 * (size_t)ths->local_N_total);
}

extern "C" void pnfft_init(void) {}
extern "C" void pnfft_cleanup(void) {}

// ===========================================================================
// memory
// ===========================================================================
extern "C" void *pnfft_malloc(size_t n) {
  void *p = engine_host_alloc(n);
  if (p) return p;
  if (n == 0) return NULL;
  if (posix_memalign(&p, 64, n) != 0) return NULL;
  return p;
}
extern "C" double *pnfft_alloc_real(size_t n) { return (double *)pnfft_malloc(sizeof(double) * n); }
extern "C" pnfft_complex *pnfft_alloc_complex(size_t n) {
  return (pnfft_complex *)pnfft_malloc(sizeof(double) * 2 * n);
}
extern "C" void pnfft_free(void *p) {
  if (!p) return;
  if (!engine_host_free(p)) free(p);
}

// ===========================================================================
// test-input generators
// ===========================================================================
// f_hat initialisation for tests.  The reference forwards to PFFT's
// init_input_complex_3d (api-basic.c:663-679), which is not part of the
// reference tree; this deterministic closed form is used instead:
//   f_hat[k] = 1000/(2g+1) + i 1000/(2g+2), g = row-major index of k + N/2.
extern "C" void pnfft_init_f_hat_3d(const ptrdiff_t *N, const ptrdiff_t *local_N, const ptrdiff_t *local_N_start,
                                    unsigned pnfft_flags, pnfft_complex *data) {
  double *d = (double *)data;
  int tr = (pnfft_flags & PNFFT_TRANSPOSED_F_HAT) ? 1 : 0;
  int64_t q = 0;
  if (tr) {
    for (ptrdiff_t k1 = local_N_start[1]; k1 < local_N_start[1] + local_N[1]; k1++)
      for (ptrdiff_t k2 = local_N_start[2]; k2 < local_N_start[2] + local_N[2]; k2++)
        for (ptrdiff_t k0 = local_N_start[0]; k0 < local_N_start[0] + local_N[0]; k0++, q++) {
          double g = (double)(((k0 + N[0] / 2) * N[1] + (k1 + N[1] / 2)) * N[2] + (k2 + N[2] / 2));
          d[2 * q] = 1000.0 / (2 * g + 1);
          d[2 * q + 1] = 1000.0 / (2 * g + 2);
        }
  } else {
    for (ptrdiff_t k0 = local_N_start[0]; k0 < local_N_start[0] + local_N[0]; k0++)
      for (ptrdiff_t k1 = local_N_start[1]; k1 < local_N_start[1] + local_N[1]; k1++)
        for (ptrdiff_t k2 = local_N_start[2]; k2 < local_N_start[2] + local_N[2]; k2++, q++) {
          double g = (double)(((k0 + N[0] / 2) * N[1] + (k1 + N[1] / 2)) * N[2] + (k2 + N[2] / 2));
          d[2 * q] = 1000.0 / (2 * g + 1);
          d[2 * q + 1] = 1000.0 / (2 * g + 2);
        }
  }
}

extern "C" void pnfft_init_f(ptrdiff_t local_M, pnfft_complex *data) {  // api-basic.c:681-691
  double *d = (double *)data;
  for (ptrdiff_t j = 0; j < local_M; j++) {
    double re = 100.0 * (double)rand() / RAND_MAX;
    double im = 100.0 * (double)rand() / RAND_MAX;
    d[2 * j] = re;
    d[2 * j + 1] = im;
  }
}

static double random_number_less_than_one(void) {  // api-adv.c:73-86
  double t;
  do {
    int it = rand();
    t = (double)it / RAND_MAX;
  } while (t >= 1.0);
  return t;
}

extern "C" void pnfft_init_x_3d_adv(const double *lo, const double *up, const double *x_max, ptrdiff_t loc_M,
                                    double *x) {  // api-adv.c:35-70
  for (int t = 0; t < 3; t++)
    if (lo[t] < -x_max[t] || x_max[t] < up[t]) return;
  for (ptrdiff_t j = 0; j < loc_M; j++)
    for (int t = 0; t < 3; t++) {
      double v;
      do {
        v = random_number_less_than_one();
        v = (up[t] - lo[t]) * v + lo[t];
      } while (v < -x_max[t] || x_max[t] <= v);
      x[3 * j + t] = v;
    }
}

extern "C" void pnfft_init_x_3d(const double *lo, const double *up, ptrdiff_t loc_M, double *x) {
  const double xm[3] = {0.5, 0.5, 0.5};
  pnfft_init_x_3d_adv(lo, up, xm, loc_M, x);
}

// ===========================================================================
// window functions (host, FP64)
// ===========================================================================
extern "C" double pnfft_inv_phi_hat(const pnfft_plan ths, int dim, ptrdiff_t k) {
  return inv_phi_hat_host(ths, dim, k);
}
extern "C" double pnfft_phi_hat(const pnfft_plan ths, int dim, ptrdiff_t k) { return phi_hat_host(ths, dim, k); }
extern "C" double pnfft_psi(const pnfft_plan ths, int dim, double x) { return window_host(ths, dim, x, 0); }
extern "C" double pnfft_dpsi(const pnfft_plan ths, int dim, double x) { return window_host(ths, dim, x, 1); }
extern "C" double pnfft_ddpsi(const pnfft_plan ths, int dim, double x) { return window_host(ths, dim, x, 2); }

// ===========================================================================
// printing (api-basic.c:705-818)
// ===========================================================================
extern "C" void pnfft_vpr_complex(pnfft_complex *data, ptrdiff_t N, const char *name, MPI_Comm) {
  if (N < 1) return;
  const double *d = (const double *)data;
  printf("\nRank 0, %s", name);
  for (ptrdiff_t l = 0; l < N; l++) {
    if (l % 4 == 0) printf("\n%4td.", l / 4);
    printf(" %.2e+%.2ei,", d[2 * l], d[2 * l + 1]);
  }
  printf("\n");
  fflush(stdout);
}

extern "C" void pnfft_vpr_real(double *data, ptrdiff_t N, const char *name, MPI_Comm) {
  if (N < 1) return;
  printf("\nRank 0, %s", name);
  for (ptrdiff_t l = 0; l < N; l++) {
    if (l % 8 == 0) printf("\n%4td.", l / 8);
    printf(" %e,", data[l]);
  }
  printf("\n");
  fflush(stdout);
}

static void apr_3d(const double *data, const ptrdiff_t *local_N, const ptrdiff_t *local_N_start, unsigned flags,
                   const char *name, int cplx) {
  int shift = (flags & PNFFT_TRANSPOSED_F_HAT) ? 1 : 0;
  ptrdiff_t n[3], s[3];
  for (int t = 0; t < 3; t++) {
    n[t] = local_N[(t + shift) % 3];
    s[t] = local_N_start[(t + shift) % 3];
  }
  printf("\n%s\n", name);
  int64_t q = 0;
  for (ptrdiff_t a = 0; a < n[0]; a++)
    for (ptrdiff_t b = 0; b < n[1]; b++) {
      printf("(%td, %td, %td..%td):", a + s[0], b + s[1], s[2], s[2] + n[2] - 1);
      for (ptrdiff_t c = 0; c < n[2]; c++, q++) {
        if (cplx) printf(" %.2e%+.2ei", data[2 * q], data[2 * q + 1]);
        else printf(" %.2e", data[q]);
      }
      printf("\n");
    }
  fflush(stdout);
}

extern "C" void pnfft_apr_complex_3d(pnfft_complex *data, ptrdiff_t *local_N, ptrdiff_t *local_N_start,
                                     unsigned flags, const char *name, MPI_Comm) {
  apr_3d((const double *)data, local_N, local_N_start, flags, name, 1);
}
extern "C" void pnfft_apr_real_3d(double *data, ptrdiff_t *local_N, ptrdiff_t *local_N_start, unsigned flags,
                                  const char *name, MPI_Comm) {
  apr_3d(data, local_N, local_N_start, flags, name, 0);
}

// ===========================================================================
// timers (kernel/timer.c)
// ===========================================================================
extern "C" double *pnfft_timer_copy(const double *orig) {
  double *c = (double *)malloc(sizeof(double) * PNFFT_TIMER_LENGTH);
  for (int t = 0; t < PNFFT_TIMER_LENGTH; t++) c[t] = orig[t];
  return c;
}
extern "C" double *pnfft_get_timer_trafo(pnfft_plan ths) {
  engine_flush_timers(ths);
  return pnfft_timer_copy(ths->timer_trafo);
}
extern "C" double *pnfft_get_timer_adj(pnfft_plan ths) {
  engine_flush_timers(ths);
  return pnfft_timer_copy(ths->timer_adj);
}
extern "C" void pnfft_timer_average(double *timer) {
  if (timer[PNFFT_TIMER_ITER] < 1.0) return;
  for (int t = 1; t < PNFFT_TIMER_LENGTH; t++) timer[t] /= timer[0];
}
extern "C" double *pnfft_timer_reduce_max(MPI_Comm, double *timer) { return pnfft_timer_copy(timer); }
extern "C" double *pnfft_timer_add(const double *a, const double *b) {
  double *s = (double *)malloc(sizeof(double) * PNFFT_TIMER_LENGTH);
  for (int t = 0; t < PNFFT_TIMER_LENGTH; t++) s[t] = a[t] + b[t];
  return s;
}
extern "C" void pnfft_timer_free(double *ths) { free(ths); }
extern "C" void pnfft_reset_timer(pnfft_plan ths) {
  engine_flush_timers(ths);
  for (int t = 0; t < PNFFT_TIMER_LENGTH; t++) ths->timer_trafo[t] = ths->timer_adj[t] = 0;
}

static const char *k_timer_names[PNFFT_TIMER_LENGTH] = {"iter",    "whole",    "loop_B",   "sort_nodes", "gcells",
                                                        "matrix_B", "matrix_F", "matrix_D", "shift_in",   "shift_out"};

static void fprint_timer(FILE *f, const char *prefix, const double *tm, int adv) {
  double avg[PNFFT_TIMER_LENGTH];
  for (int t = 0; t < PNFFT_TIMER_LENGTH; t++) avg[t] = tm[t];
  pnfft_timer_average(avg);
  fprintf(f, "%s(%d) = %.6e;  %% average of %d calls, seconds\n", prefix, PNFFT_TIMER_WHOLE, avg[PNFFT_TIMER_WHOLE],
          (int)tm[PNFFT_TIMER_ITER]);
  if (!adv) return;
  for (int t = 2; t < PNFFT_TIMER_LENGTH; t++)
    fprintf(f, "%s(%d) = %.6e;  %% %s\n", prefix, t, avg[t], k_timer_names[t]);
}

static void fprint_plan_timers(FILE *f, const pnfft_plan ths, int adv) {
  engine_flush_timers(ths);
  fprintf(f, "%% PNFFT (libpnfft_gb300) N=[%td %td %td] n=[%td %td %td] m=%d precision=%s\n", (ptrdiff_t)ths->N[0],
          (ptrdiff_t)ths->N[1], (ptrdiff_t)ths->N[2], (ptrdiff_t)ths->n[0], (ptrdiff_t)ths->n[1], (ptrdiff_t)ths->n[2],
          ths->m, ths->precision == PNFFT_GB300_FP32_MIXED ? "fp32-mixed" : "fp64");
  fprint_timer(f, "pnfft_trafo", ths->timer_trafo, adv);
  fprint_timer(f, "pnfft_adj", ths->timer_adj, adv);
}

extern "C" void pnfft_print_average_timer(const pnfft_plan ths, MPI_Comm) { fprint_plan_timers(stdout, ths, 0); }
extern "C" void pnfft_print_average_timer_adv(const pnfft_plan ths, MPI_Comm) { fprint_plan_timers(stdout, ths, 1); }
extern "C" void pnfft_write_average_timer(const pnfft_plan ths, const char *name, MPI_Comm) {
  FILE *f = fopen(name, "a+");
  if (!f) {
    fprintf(stderr, "Error: Cannot open file %s.\n", name);
    return;
  }
  fprint_plan_timers(f, ths, 0);
  fclose(f);
}
extern "C" void pnfft_write_average_timer_adv(const pnfft_plan ths, const char *name, MPI_Comm) {
  FILE *f = fopen(name, "a+");
  if (!f) {
    fprintf(stderr, "Error: Cannot open file %s.\n", name);
    return;
  }
  fprint_plan_timers(f, ths, 1);
  fclose(f);
}

// ===========================================================================
// command line (util/getargs.c, api-basic.c:820-953)
// ===========================================================================
extern "C" void pnfft_get_args(int argc, char **argv, const char *name, int neededArgs, unsigned type,
                               void *parameter) {
  for (int i = 1; i < argc; i++) {
    if (strcmp(argv[i], name) != 0) continue;
    if (i + neededArgs >= argc) {
      fprintf(stderr, "Error: option %s needs %d argument(s)\n", name, neededArgs);
      return;
    }
    for (int k = 0; k < neededArgs; k++) {
      const char *v = argv[i + 1 + k];
      switch (type) {
        case PFFT_INT: ((int *)parameter)[k] = atoi(v); break;
        case PFFT_PTRDIFF_T: ((ptrdiff_t *)parameter)[k] = (ptrdiff_t)atoll(v); break;
        case PFFT_FLOAT: ((float *)parameter)[k] = (float)atof(v); break;
        case PFFT_DOUBLE: ((double *)parameter)[k] = atof(v); break;
        case PFFT_LDOUBLE: ((long double *)parameter)[k] = (long double)atof(v); break;
        case PFFT_UNSIGNED: ((unsigned *)parameter)[k] = (unsigned)strtoul(v, NULL, 10); break;
        default: break;
      }
    }
    return;
  }
}

extern "C" void pnfft_check_init_parameters(int argc, char **argv, ptrdiff_t *N, ptrdiff_t *n, ptrdiff_t *local_M,
                                            int *m, unsigned *pnfft_flags, unsigned *compute_flags, double *x_max,
                                            int *np, int *compare_direct, int *debug) {
  int window = 4, fast_gaussian = 0, intpol = -1, interlaced = 0, diff_ik = 0, tr_f_hat = 0;
  int compute_f = 1, compute_grad_f = 1, compute_hessian_f = 1;
  N[0] = N[1] = N[2] = 16;
  n[0] = n[1] = n[2] = 0;
  *local_M = 0;
  *m = 6;
  x_max[0] = x_max[1] = x_max[2] = 0.5;
  np[0] = 1;
  np[1] = 1;
  np[2] = 1;
  pnfft_get_args(argc, argv, "-pnfft_local_M", 1, PFFT_PTRDIFF_T, local_M);
  pnfft_get_args(argc, argv, "-pnfft_N", 3, PFFT_PTRDIFF_T, N);
  pnfft_get_args(argc, argv, "-pnfft_n", 3, PFFT_PTRDIFF_T, n);
  pnfft_get_args(argc, argv, "-pnfft_np", 3, PFFT_INT, np);
  pnfft_get_args(argc, argv, "-pnfft_m", 1, PFFT_INT, m);
  pnfft_get_args(argc, argv, "-pnfft_window", 1, PFFT_INT, &window);
  pnfft_get_args(argc, argv, "-pnfft_fast_gaussian", 1, PFFT_INT, &fast_gaussian);
  pnfft_get_args(argc, argv, "-pnfft_intpol", 1, PFFT_INT, &intpol);
  pnfft_get_args(argc, argv, "-pnfft_interlaced", 1, PFFT_INT, &interlaced);
  pnfft_get_args(argc, argv, "-pnfft_diff_ik", 1, PFFT_INT, &diff_ik);
  pnfft_get_args(argc, argv, "-pnfft_tr_f_hat", 1, PFFT_INT, &tr_f_hat);
  pnfft_get_args(argc, argv, "-pnfft_x_max", 3, PFFT_DOUBLE, x_max);
  pnfft_get_args(argc, argv, "-pnfft_debug", 1, PFFT_INT, debug);
  pnfft_get_args(argc, argv, "-pnfft_compare_direct", 1, PFFT_INT, compare_direct);
  pnfft_get_args(argc, argv, "-pnfft_compute_f", 1, PFFT_INT, &compute_f);
  pnfft_get_args(argc, argv, "-pnfft_compute_grad_f", 1, PFFT_INT, &compute_grad_f);
  pnfft_get_args(argc, argv, "-pnfft_compute_hessian_f", 1, PFFT_INT, &compute_hessian_f);
  if (*local_M == 0) *local_M = N[0] * N[1] * N[2] / ((ptrdiff_t)np[0] * np[1] * np[2]);
  for (int t = 0; t < 3; t++)
    if (n[t] == 0) n[t] = 2 * N[t];
  unsigned wf;
  switch (window) {
    case 0: wf = PNFFT_WINDOW_GAUSSIAN; break;
    case 1: wf = PNFFT_WINDOW_BSPLINE; break;
    case 2: wf = PNFFT_WINDOW_SINC_POWER; break;
    case 3: wf = PNFFT_WINDOW_BESSEL_I0; break;
    case 5: wf = PNFFT_WINDOW_GAUSSIAN_T; break;
    default: wf = PNFFT_WINDOW_KAISER_BESSEL;
  }
  unsigned ipf = 0;
  switch (intpol) {
    case 0: ipf = PNFFT_PRE_CONST_PSI; break;
    case 1: ipf = PNFFT_PRE_LIN_PSI; break;
    case 2: ipf = PNFFT_PRE_QUAD_PSI; break;
    case 3: ipf = PNFFT_PRE_CUB_PSI; break;
    default: ipf = 0;
  }
  *compute_flags = 0;
  if (compute_f) *compute_flags |= PNFFT_COMPUTE_F;
  if (compute_grad_f) *compute_flags |= PNFFT_COMPUTE_GRAD_F;
  if (compute_hessian_f) *compute_flags |= PNFFT_COMPUTE_HESSIAN_F;
  printf("* Computation of parallel NFFT (libpnfft_gb300, one GPU)\n");
  printf("* for  N = %td x %td x %td Fourier coefficients, local_M = %td nodes, n = %td x %td x %td, m = %d,\n", N[0],
         N[1], N[2], *local_M, n[0], n[1], n[2], *m);
  printf("*      window = %d, fast Gaussian = %d, intpol = %d, interlaced = %d, diff_ik = %d, tr_f_hat = %d\n", window,
         fast_gaussian, intpol, interlaced, diff_ik, tr_f_hat);
  *pnfft_flags = wf | (fast_gaussian ? PNFFT_FAST_GAUSSIAN : 0u) | ipf | (diff_ik ? PNFFT_DIFF_IK : 0u) |
                 (tr_f_hat ? PNFFT_TRANSPOSED_F_HAT : 0u) | (interlaced ? PNFFT_INTERLACED : 0u);
}

// ===========================================================================
// extensions (include/pnfft_gb300.h)
// ===========================================================================
extern "C" const char *pnfft_gb300_last_error(void) { return last_error(); }
extern "C" void pnfft_gb300_clear_error(void) { g_err.clear(); }
extern "C" int pnfft_gb300_device_count(void) { return engine_device_count(); }

extern "C" int pnfft_gb300_set_precision(pnfft_plan ths, int precision) {
  if (!ths) return -1;
  if (precision != PNFFT_GB300_FP64 && precision != PNFFT_GB300_FP32_MIXED) {
    set_error("pnfft_gb300_set_precision: unknown precision %d", precision);
    return -1;
  }
  if (precision == PNFFT_GB300_FP32_MIXED && !fp32_window_in_range(ths)) return -1;
  if (ths->precision != precision) {
    engine_sync(ths);
    ths->precision = precision;
    ths->table_version++;
  }
  return 0;
}
extern "C" int pnfft_gb300_get_precision(const pnfft_plan ths) { return ths ? ths->precision : -1; }
extern "C" int pnfft_gb300_set_conv_method(pnfft_plan ths, int method) {
  if (!ths) return -1;
  if (method < 0 || method > 3) {
    set_error("pnfft_gb300_set_conv_method: unknown method %d (0: lines / tiles, 1: per node, 2: one warp per "
              "node, 3: grouped)",
              method);
    return -1;
  }
  ths->conv_method[0] = ths->conv_method[1] = method;
  return 0;
}
extern "C" int pnfft_gb300_get_conv_method(const pnfft_plan ths) { return ths ? ths->conv_method[0] : -1; }
extern "C" int pnfft_gb300_get_tuning(const pnfft_plan ths, int *tuning) {
  if (!ths || !tuning) return -1;
  tuning[0] = ths->conv_method[0];
  tuning[1] = ths->conv_method[1];
  tuning[2] = ths->line_sub_max;
  return 0;
}
extern "C" int pnfft_gb300_set_tuning(pnfft_plan ths, const int *tuning) {
  if (!ths || !tuning) return -1;
  for (int d = 0; d < 2; d++)
    if (tuning[d] < 0 || tuning[d] > 3) {
      set_error("pnfft_gb300_set_tuning: unknown method %d", tuning[d]);
      return -1;
    }
  if (tuning[2] < 32 || tuning[2] > 4096 || (tuning[2] & 31)) {
    set_error("pnfft_gb300_set_tuning: nodes per line sub-problem %d not a multiple of 32 in [32, 4096]", tuning[2]);
    return -1;
  }
  ths->conv_method[0] = tuning[0];
  ths->conv_method[1] = tuning[1];
  ths->line_sub_max = tuning[2];
  return 0;
}
extern "C" int pnfft_gb300_autotune(pnfft_plan ths, pnfft_nodes nodes, unsigned trafo_flags, unsigned adj_flags,
                                    int reps) {
  if (!ths || !nodes) {
    set_error("pnfft_gb300_autotune: plan and nodes are required");
    return -1;
  }
  return engine_autotune(ths, nodes, trafo_flags, adj_flags, reps > 0 ? reps : 2);
}
extern "C" int pnfft_gb300_batch_begin(void *stream) { return engine_batch_begin(stream); }
extern "C" int pnfft_gb300_batch_end(void) { return engine_batch_end(); }
extern "C" int pnfft_gb300_batch_stats(int *deferred_calls, int *launches) {
  if (!deferred_calls || !launches) return -1;
  engine_batch_stats(deferred_calls, launches);
  return 0;
}
extern "C" int pnfft_gb300_get_conv_kernel(const pnfft_plan ths, int adjoint) {
  return ths ? ths->last_conv[adjoint ? 1 : 0] : -1;
}
extern "C" int pnfft_gb300_set_stream(pnfft_plan ths, void *stream) { return ths ? engine_set_stream(ths, stream) : -1; }
extern "C" int pnfft_gb300_set_device_f_hat(pnfft_plan ths, void *d) {
  if (!ths) return -1;
  ths->d_f_hat_user = d;
  return 0;
}
extern "C" int pnfft_gb300_set_device_arrays(pnfft_nodes nodes, double *d_x, void *d_f, void *d_grad_f,
                                             void *d_hessian_f) {
  if (!nodes) return -1;
  if (nodes->u_x != d_x) nodes->version++;
  nodes->u_x = d_x;
  nodes->u_f = d_f;
  nodes->u_grad = d_grad_f;
  nodes->u_hess = d_hessian_f;
  return 0;
}
extern "C" int pnfft_gb300_nodes_set_fixed(pnfft_nodes nodes, int fixed) {
  if (!nodes) return -1;
  nodes->fixed = fixed ? 1 : 0;
  nodes->version++;
  return 0;
}
extern "C" int pnfft_gb300_synchronize(pnfft_plan ths) { return ths ? engine_sync(ths) : -1; }
extern "C" int pnfft_gb300_sort_nodes(pnfft_plan ths, ptrdiff_t M, const double *x, long long *pairs) {
  if (!ths) return -1;
  return engine_sort_nodes(ths, M, x, pairs);
}
extern "C" int pnfft_gb300_node_index(pnfft_plan ths, ptrdiff_t M, const double *x, int interlaced, long long *u) {
  if (!ths) return -1;
  return engine_node_index(ths, M, x, interlaced, u);
}
extern "C" int pnfft_gb300_last_stage_ms(const pnfft_plan ths, int adjoint, double *ms10) {
  if (!ths) return -1;
  engine_flush_timers(ths);
  for (int t = 0; t < PNFFT_TIMER_LENGTH; t++) ms10[t] = ths->last_ms[adjoint ? 1 : 0][t];
  return 0;
}
