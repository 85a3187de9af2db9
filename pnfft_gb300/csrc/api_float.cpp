// api_float.cpp -- the single-precision API pnfftf_* (the float expansion of
// PNFFT_DEFINE_API, api/pnfft.h:287) as a layer over the double library.
//
// A float plan wraps a double plan and runs in the FP32-mixed precision of the
// GPU path (FP64 when the window would overflow FP32); float nodes wrap double
// nodes.  pnfftf_trafo / pnfftf_adj (float_io.cu) copy the caller's float
// arrays to the GPU, widen them there, run the double plan on those device
// arrays and round the outputs to float on the GPU before copying them back.
// Ownership and flag semantics are those of the double API (api-basic.c:402-442).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/pnfft.h"
#include "api_float.h"

namespace {

void to_double(double *d, const float *s, size_t n) {
  for (size_t i = 0; i < n; i++) d[i] = (double)s[i];
}

pnfftf_plan wrap(pnfft_plan p, int c2r, unsigned pnfft_flags, const ptrdiff_t *local_N) {
  if (!p) return nullptr;
  pnfftf_plan f = (pnfftf_plan)calloc(1, sizeof(pnfftf_plan_s));
  f->p = p;
  f->c2r = c2r;
  f->nfh = local_N[0] * local_N[1] * local_N[2];
  if (pnfft_flags & PNFFT_MALLOC_F_HAT) {
    f->f_hat = (float *)pnfft_malloc(sizeof(float) * 2 * (size_t)f->nfh);
    if (f->f_hat) memset(f->f_hat, 0, sizeof(float) * 2 * (size_t)f->nfh);
    f->own_f_hat = 1;
  }
  // the float API computes in the FP32-mixed form unless the window overflows it
  if (pnfft_gb300_set_precision(p, PNFFT_GB300_FP32_MIXED) != 0) pnfft_gb300_clear_error();
  return f;
}

void xmax_d(const float *x_max, double *d) {
  for (int t = 0; t < 3; t++) d[t] = (double)x_max[t];
}

// sizes of the stored arrays of a transform on these nodes
size_t tuple(pnfftf_plan ths) { return ths->c2r ? 1 : 2; }

}  // namespace

extern "C" {

int pnfftf_create_procmesh_2d(MPI_Comm comm, int np0, int np1, MPI_Comm *comm_cart_2d) {
  return pnfft_create_procmesh_2d(comm, np0, np1, comm_cart_2d);
}
int pnfftf_create_procmesh(int rnk, MPI_Comm comm, const int *np, MPI_Comm *comm_cart) {
  return pnfft_create_procmesh(rnk, comm, np, comm_cart);
}

// --- local sizes -------------------------------------------------------------
#define PG_BORDERS_TO_FLOAT                                   \
  for (int t = 0; t < 3; t++) {                               \
    lower_border[t] = (float)lo[t];                           \
    upper_border[t] = (float)up[t];                           \
  }

void pnfftf_local_size_3d(const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                          ptrdiff_t *local_N_start, float *lower_border, float *upper_border) {
  double lo[3], up[3];
  pnfft_local_size_3d(N, comm_cart, pnfft_flags, local_N, local_N_start, lo, up);
  PG_BORDERS_TO_FLOAT
}
void pnfftf_local_size_3d_c2r(const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                              ptrdiff_t *local_N_start, float *lower_border, float *upper_border) {
  double lo[3], up[3];
  pnfft_local_size_3d_c2r(N, comm_cart, pnfft_flags, local_N, local_N_start, lo, up);
  PG_BORDERS_TO_FLOAT
}
void pnfftf_local_size_adv(int d, const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                           ptrdiff_t *local_N_start, float *lower_border, float *upper_border) {
  double lo[3], up[3];
  pnfft_local_size_adv(d, N, comm_cart, pnfft_flags, local_N, local_N_start, lo, up);
  PG_BORDERS_TO_FLOAT
}
void pnfftf_local_size_adv_c2r(int d, const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags,
                               ptrdiff_t *local_N, ptrdiff_t *local_N_start, float *lower_border,
                               float *upper_border) {
  double lo[3], up[3];
  pnfft_local_size_adv_c2r(d, N, comm_cart, pnfft_flags, local_N, local_N_start, lo, up);
  PG_BORDERS_TO_FLOAT
}
void pnfftf_local_size_guru(int d, const ptrdiff_t *N, const ptrdiff_t *n, const float *x_max, int m,
                            MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N, ptrdiff_t *local_N_start,
                            float *lower_border, float *upper_border) {
  double lo[3], up[3], xm[3];
  xmax_d(x_max, xm);
  pnfft_local_size_guru(d, N, n, xm, m, comm_cart, pnfft_flags, local_N, local_N_start, lo, up);
  PG_BORDERS_TO_FLOAT
}
void pnfftf_local_size_guru_c2r(int d, const ptrdiff_t *N, const ptrdiff_t *n, const float *x_max, int m,
                                MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                                ptrdiff_t *local_N_start, float *lower_border, float *upper_border) {
  double lo[3], up[3], xm[3];
  xmax_d(x_max, xm);
  pnfft_local_size_guru_c2r(d, N, n, xm, m, comm_cart, pnfft_flags, local_N, local_N_start, lo, up);
  PG_BORDERS_TO_FLOAT
}
#undef PG_BORDERS_TO_FLOAT

// --- plans ---------------------------------------------------------------------
pnfftf_plan pnfftf_init_3d(const ptrdiff_t *N, MPI_Comm comm_cart) {
  ptrdiff_t ln[3], ls[3];
  double lo[3], up[3];
  pnfft_local_size_3d(N, comm_cart, 0, ln, ls, lo, up);
  return wrap(pnfft_init_3d(N, comm_cart), 0, PNFFT_MALLOC_F_HAT, ln);
}
pnfftf_plan pnfftf_init_3d_c2r(const ptrdiff_t *N, MPI_Comm comm_cart) {
  ptrdiff_t ln[3], ls[3];
  double lo[3], up[3];
  pnfft_local_size_3d_c2r(N, comm_cart, 0, ln, ls, lo, up);
  return wrap(pnfft_init_3d_c2r(N, comm_cart), 1, PNFFT_MALLOC_F_HAT, ln);
}
pnfftf_plan pnfftf_init_adv(int d, const ptrdiff_t *N, unsigned pnfft_flags, unsigned pfft_flags,
                            MPI_Comm comm_cart) {
  ptrdiff_t ln[3], ls[3];
  double lo[3], up[3];
  pnfft_local_size_adv(d, N, comm_cart, pnfft_flags, ln, ls, lo, up);
  return wrap(pnfft_init_adv(d, N, pnfft_flags | PNFFT_MALLOC_F_HAT, pfft_flags, comm_cart), 0, pnfft_flags, ln);
}
pnfftf_plan pnfftf_init_adv_c2r(int d, const ptrdiff_t *N, unsigned pnfft_flags, unsigned pfft_flags,
                                MPI_Comm comm_cart) {
  ptrdiff_t ln[3], ls[3];
  double lo[3], up[3];
  pnfft_local_size_adv_c2r(d, N, comm_cart, pnfft_flags, ln, ls, lo, up);
  return wrap(pnfft_init_adv_c2r(d, N, pnfft_flags | PNFFT_MALLOC_F_HAT, pfft_flags, comm_cart), 1, pnfft_flags,
              ln);
}
pnfftf_plan pnfftf_init_guru(int d, const ptrdiff_t *N, const ptrdiff_t *n, const float *x_max, int m,
                             unsigned pnfft_flags, unsigned pfft_flags, MPI_Comm comm_cart) {
  ptrdiff_t ln[3], ls[3];
  double lo[3], up[3], xm[3];
  xmax_d(x_max, xm);
  pnfft_local_size_guru(d, N, n, xm, m, comm_cart, pnfft_flags, ln, ls, lo, up);
  return wrap(pnfft_init_guru(d, N, n, xm, m, pnfft_flags | PNFFT_MALLOC_F_HAT, pfft_flags, comm_cart), 0,
              pnfft_flags, ln);
}
pnfftf_plan pnfftf_init_guru_c2r(int d, const ptrdiff_t *N, const ptrdiff_t *n, const float *x_max, int m,
                                 unsigned pnfft_flags, unsigned pfft_flags, MPI_Comm comm_cart) {
  ptrdiff_t ln[3], ls[3];
  double lo[3], up[3], xm[3];
  xmax_d(x_max, xm);
  pnfft_local_size_guru_c2r(d, N, n, xm, m, comm_cart, pnfft_flags, ln, ls, lo, up);
  return wrap(pnfft_init_guru_c2r(d, N, n, xm, m, pnfft_flags | PNFFT_MALLOC_F_HAT, pfft_flags, comm_cart), 1,
              pnfft_flags, ln);
}

pnfft_plan pnfftf_gb300_double_plan(pnfftf_plan ths) { return ths ? ths->p : nullptr; }

void pnfftf_finalize(pnfftf_plan ths, unsigned pnfft_finalize_flags) {
  if (!ths) return;
  if ((pnfft_finalize_flags & PNFFT_FREE_F_HAT) && ths->f_hat) pnfft_free(ths->f_hat);
  pnfft_finalize(ths->p, PNFFT_FREE_F_HAT);  // synchronizes the plan's stream
  pg::float_dev_free(ths->dev);
  free(ths);
}

// --- nodes ---------------------------------------------------------------------
pnfftf_nodes pnfftf_init_nodes(ptrdiff_t local_M, unsigned malloc_flags) {
  pnfftf_nodes n = (pnfftf_nodes)calloc(1, sizeof(pnfftf_nodes_s));
  n->M = local_M;
  n->nd = pnfft_init_nodes(local_M, 0);
  const size_t M = (size_t)(local_M > 0 ? local_M : 0);
  if (malloc_flags & PNFFT_MALLOC_X) n->x = pnfftf_alloc_real(3 * M);
  if (malloc_flags & PNFFT_MALLOC_F) n->f = (float *)pnfftf_alloc_complex(M);
  if (malloc_flags & PNFFT_MALLOC_GRAD_F) n->grad = (float *)pnfftf_alloc_complex(3 * M);
  if (malloc_flags & PNFFT_MALLOC_HESSIAN_F) n->hess = (float *)pnfftf_alloc_complex(6 * M);
  return n;
}

void pnfftf_free_nodes(pnfftf_nodes nodes, unsigned pnfft_finalize_flags) {
  if (!nodes) return;
  if ((pnfft_finalize_flags & PNFFT_FREE_X) && nodes->x) pnfft_free(nodes->x);
  if ((pnfft_finalize_flags & PNFFT_FREE_F) && nodes->f) pnfft_free(nodes->f);
  if ((pnfft_finalize_flags & PNFFT_FREE_GRAD_F) && nodes->grad) pnfft_free(nodes->grad);
  if ((pnfft_finalize_flags & PNFFT_FREE_HESSIAN_F) && nodes->hess) pnfft_free(nodes->hess);
  pnfft_free_nodes(nodes->nd, 0);
  pg::float_dev_free(nodes->dev);
  free(nodes);
}

// the window values are evaluated on the fly (pnfft_precompute_psi); what
// the call keeps is the promise that the coordinates stay fixed
void pnfftf_precompute_psi(pnfftf_plan ths, pnfftf_nodes nodes, unsigned precompute_flags) {
  if (!ths || !nodes) return;
  pnfft_precompute_psi(ths->p, nodes->nd, precompute_flags);
}

// --- setters / getters -----------------------------------------------------------
void pnfftf_set_f(pnfftf_complex *f, pnfftf_nodes nodes) { nodes->f = (float *)f; }
void pnfftf_set_grad_f(pnfftf_complex *grad_f, pnfftf_nodes nodes) { nodes->grad = (float *)grad_f; }
void pnfftf_set_hessian_f(pnfftf_complex *hessian_f, pnfftf_nodes nodes) { nodes->hess = (float *)hessian_f; }
void pnfftf_set_f_real(float *f, pnfftf_nodes nodes) { nodes->f = f; }
void pnfftf_set_grad_f_real(float *grad_f, pnfftf_nodes nodes) { nodes->grad = grad_f; }
void pnfftf_set_hessian_f_real(float *hessian_f, pnfftf_nodes nodes) { nodes->hess = hessian_f; }
void pnfftf_set_x(float *x, pnfftf_nodes nodes) { nodes->x = x; }
void pnfftf_set_f_hat(pnfftf_complex *f_hat, pnfftf_plan ths) { ths->f_hat = (float *)f_hat; }
void pnfftf_set_f_hat_real(float *f_hat, pnfftf_plan ths) { ths->f_hat = f_hat; }
void pnfftf_set_b(float b0, float b1, float b2, pnfftf_plan ths) { pnfft_set_b(b0, b1, b2, ths->p); }

pnfftf_complex *pnfftf_get_f(const pnfftf_nodes nodes) { return (pnfftf_complex *)nodes->f; }
pnfftf_complex *pnfftf_get_grad_f(const pnfftf_nodes nodes) { return (pnfftf_complex *)nodes->grad; }
pnfftf_complex *pnfftf_get_hessian_f(const pnfftf_nodes nodes) { return (pnfftf_complex *)nodes->hess; }
float *pnfftf_get_f_real(const pnfftf_nodes nodes) { return nodes->f; }
float *pnfftf_get_grad_f_real(const pnfftf_nodes nodes) { return nodes->grad; }
float *pnfftf_get_hessian_f_real(const pnfftf_nodes nodes) { return nodes->hess; }
float *pnfftf_get_x(const pnfftf_nodes nodes) { return nodes->x; }
pnfftf_complex *pnfftf_get_f_hat(const pnfftf_plan ths) { return (pnfftf_complex *)ths->f_hat; }
float *pnfftf_get_f_hat_real(const pnfftf_plan ths) { return ths->f_hat; }
int pnfftf_get_d(const pnfftf_plan ths) { return pnfft_get_d(ths->p); }
int pnfftf_get_m(const pnfftf_plan ths) { return pnfft_get_m(ths->p); }
void pnfftf_get_x_max(const pnfftf_plan ths, float *x_max) {
  double d[3];
  pnfft_get_x_max(ths->p, d);
  for (int t = 0; t < 3; t++) x_max[t] = (float)d[t];
}
void pnfftf_get_N(const pnfftf_plan ths, ptrdiff_t *N) { pnfft_get_N(ths->p, N); }
void pnfftf_get_n(const pnfftf_plan ths, ptrdiff_t *n) { pnfft_get_n(ths->p, n); }
unsigned pnfftf_get_pnfft_flags(const pnfftf_plan ths) { return pnfft_get_pnfft_flags(ths->p); }
unsigned pnfftf_get_pfft_flags(const pnfftf_plan ths) { return pnfft_get_pfft_flags(ths->p); }
void pnfftf_get_b(const pnfftf_plan ths, float *b0, float *b1, float *b2) {
  double a0, a1, a2;
  pnfft_get_b(ths->p, &a0, &a1, &a2);
  *b0 = (float)a0;
  *b1 = (float)a1;
  *b2 = (float)a2;
}

// --- transforms ------------------------------------------------------------------
void pnfftf_trafo(pnfftf_plan ths, pnfftf_nodes nodes, unsigned compute_flags) {
  if (!ths || !nodes) return;  // api-basic.c:205-206
  if (pnfftf_gb300_trafo_dev(ths, nodes, compute_flags)) fprintf(stderr, "pnfftf_trafo: %s\n", pnfft_gb300_last_error());
}

void pnfftf_adj(pnfftf_plan ths, pnfftf_nodes nodes, unsigned compute_flags) {
  if (!ths || !nodes) return;
  if (pnfftf_gb300_adj_dev(ths, nodes, compute_flags)) fprintf(stderr, "pnfftf_adj: %s\n", pnfft_gb300_last_error());
}

// --- memory, generators ------------------------------------------------------------
void pnfftf_init(void) { pnfft_init(); }
void pnfftf_cleanup(void) { pnfft_cleanup(); }
void *pnfftf_malloc(size_t n) { return pnfft_malloc(n); }
float *pnfftf_alloc_real(size_t n) { return (float *)pnfft_malloc(sizeof(float) * n); }
pnfftf_complex *pnfftf_alloc_complex(size_t n) { return (pnfftf_complex *)pnfft_malloc(sizeof(float) * 2 * n); }
void pnfftf_free(void *p) { pnfft_free(p); }

// the deterministic stand-in of pnfft_init_f_hat_3d, evaluated in float
void pnfftf_init_f_hat_3d(const ptrdiff_t *N, const ptrdiff_t *local_N, const ptrdiff_t *local_N_start,
                          unsigned pnfft_flags, pnfftf_complex *data) {
  float *d = (float *)data;
  const int tr = (pnfft_flags & PNFFT_TRANSPOSED_F_HAT) ? 1 : 0;
  const int o[3] = {tr ? 1 : 0, tr ? 2 : 1, tr ? 0 : 2};  // loop order (outer to inner)
  ptrdiff_t k[3];
  size_t q = 0;
  for (k[o[0]] = local_N_start[o[0]]; k[o[0]] < local_N_start[o[0]] + local_N[o[0]]; k[o[0]]++)
    for (k[o[1]] = local_N_start[o[1]]; k[o[1]] < local_N_start[o[1]] + local_N[o[1]]; k[o[1]]++)
      for (k[o[2]] = local_N_start[o[2]]; k[o[2]] < local_N_start[o[2]] + local_N[o[2]]; k[o[2]]++, q++) {
        const float g = (float)(((k[0] + N[0] / 2) * N[1] + (k[1] + N[1] / 2)) * N[2] + (k[2] + N[2] / 2));
        d[2 * q] = 1000.0f / (2 * g + 1);
        d[2 * q + 1] = 1000.0f / (2 * g + 2);
      }
}

// api-basic.c:681-691 with R = float: 100.0 * (R)rand() / RAND_MAX in double, rounded to R
void pnfftf_init_f(ptrdiff_t local_M, pnfftf_complex *data) {
  float *d = (float *)data;
  for (ptrdiff_t j = 0; j < local_M; j++) {
    const float re = (float)(100.0 * (float)rand() / RAND_MAX);
    const float im = (float)(100.0 * (float)rand() / RAND_MAX);
    d[2 * j] = re;
    d[2 * j + 1] = im;
  }
}

// api-adv.c:73-86 with R = float: (R)rand() / RAND_MAX in float, below 1
static float random_number_less_than_one_f(void) {
  float t;
  do {
    const int it = rand();
    t = (float)it / RAND_MAX;
  } while (t >= 1.0f);
  return t;
}

void pnfftf_init_x_3d_adv(const float *lo, const float *up, const float *x_max, ptrdiff_t loc_M, float *x) {
  for (int t = 0; t < 3; t++)
    if (lo[t] < -x_max[t] || x_max[t] < up[t]) return;  // api-adv.c:53-64
  for (ptrdiff_t j = 0; j < loc_M; j++)
    for (int t = 0; t < 3; t++) {
      float v;
      do {
        v = random_number_less_than_one_f();
        v = (up[t] - lo[t]) * v + lo[t];
      } while (v < -x_max[t] || x_max[t] <= v);
      x[3 * j + t] = v;
    }
}
void pnfftf_init_x_3d(const float *lo, const float *up, ptrdiff_t loc_M, float *x) {
  const float xm[3] = {0.5f, 0.5f, 0.5f};
  pnfftf_init_x_3d_adv(lo, up, xm, loc_M, x);
}

void pnfftf_zero_f_hat(pnfftf_plan ths) {
  if (ths && ths->f_hat) memset(ths->f_hat, 0, sizeof(float) * 2 * (size_t)ths->nfh);
}

// --- windows --------------------------------------------------------------------
float pnfftf_inv_phi_hat(const pnfftf_plan ths, int dim, ptrdiff_t k) {
  return (float)pnfft_inv_phi_hat(ths->p, dim, k);
}
float pnfftf_phi_hat(const pnfftf_plan ths, int dim, ptrdiff_t k) { return (float)pnfft_phi_hat(ths->p, dim, k); }
float pnfftf_psi(const pnfftf_plan ths, int dim, float x) { return (float)pnfft_psi(ths->p, dim, x); }
float pnfftf_dpsi(const pnfftf_plan ths, int dim, float x) { return (float)pnfft_dpsi(ths->p, dim, x); }
float pnfftf_ddpsi(const pnfftf_plan ths, int dim, float x) { return (float)pnfft_ddpsi(ths->p, dim, x); }

// --- printing (same format as the double functions) --------------------------------
void pnfftf_vpr_complex(pnfftf_complex *data, ptrdiff_t N, const char *name, MPI_Comm comm) {
  if (N < 1) return;
  double *d = (double *)malloc(sizeof(double) * 2 * (size_t)N);
  to_double(d, (const float *)data, 2 * (size_t)N);
  pnfft_vpr_complex((pnfft_complex *)d, N, name, comm);
  free(d);
}
void pnfftf_vpr_real(float *data, ptrdiff_t N, const char *name, MPI_Comm comm) {
  if (N < 1) return;
  double *d = (double *)malloc(sizeof(double) * (size_t)N);
  to_double(d, data, (size_t)N);
  pnfft_vpr_real(d, N, name, comm);
  free(d);
}
void pnfftf_apr_complex_3d(pnfftf_complex *data, ptrdiff_t *local_N, ptrdiff_t *local_N_start,
                           unsigned pnfft_flags, const char *name, MPI_Comm comm) {
  const size_t n = (size_t)(local_N[0] * local_N[1] * local_N[2]);
  double *d = (double *)malloc(sizeof(double) * 2 * (n ? n : 1));
  to_double(d, (const float *)data, 2 * n);
  pnfft_apr_complex_3d((pnfft_complex *)d, local_N, local_N_start, pnfft_flags, name, comm);
  free(d);
}
void pnfftf_apr_real_3d(float *data, ptrdiff_t *local_N, ptrdiff_t *local_N_start, unsigned pnfft_flags,
                        const char *name, MPI_Comm comm) {
  const size_t n = (size_t)(local_N[0] * local_N[1] * local_N[2]);
  double *d = (double *)malloc(sizeof(double) * (n ? n : 1));
  to_double(d, data, n);
  pnfft_apr_real_3d(d, local_N, local_N_start, pnfft_flags, name, comm);
  free(d);
}

// --- timers (double in every precision) ------------------------------------------------
double *pnfftf_get_timer_trafo(pnfftf_plan ths) { return pnfft_get_timer_trafo(ths->p); }
double *pnfftf_get_timer_adj(pnfftf_plan ths) { return pnfft_get_timer_adj(ths->p); }
void pnfftf_timer_average(double *timer) { pnfft_timer_average(timer); }
double *pnfftf_timer_copy(const double *orig) { return pnfft_timer_copy(orig); }
double *pnfftf_timer_reduce_max(MPI_Comm comm, double *timer) { return pnfft_timer_reduce_max(comm, timer); }
double *pnfftf_timer_add(const double *sum1, const double *sum2) { return pnfft_timer_add(sum1, sum2); }
void pnfftf_timer_free(double *ths) { pnfft_timer_free(ths); }
void pnfftf_reset_timer(pnfftf_plan ths) { pnfft_reset_timer(ths->p); }
void pnfftf_print_average_timer(const pnfftf_plan ths, MPI_Comm comm) { pnfft_print_average_timer(ths->p, comm); }
void pnfftf_print_average_timer_adv(const pnfftf_plan ths, MPI_Comm comm) {
  pnfft_print_average_timer_adv(ths->p, comm);
}
void pnfftf_write_average_timer(const pnfftf_plan ths, const char *name, MPI_Comm comm) {
  pnfft_write_average_timer(ths->p, name, comm);
}
void pnfftf_write_average_timer_adv(const pnfftf_plan ths, const char *name, MPI_Comm comm) {
  pnfft_write_average_timer_adv(ths->p, name, comm);
}

void pnfftf_get_args(int argc, char **argv, const char *name, int neededArgs, unsigned type, void *parameter) {
  pnfft_get_args(argc, argv, name, neededArgs, type, parameter);
}
void pnfftf_check_init_parameters(int argc, char **argv, ptrdiff_t *N, ptrdiff_t *n, ptrdiff_t *M, int *m,
                                  unsigned *pnfft_flags, unsigned *compute_flags, double *x_max, int *np,
                                  int *compare_direct, int *debug) {
  pnfft_check_init_parameters(argc, argv, N, n, M, m, pnfft_flags, compute_flags, x_max, np, compare_direct, debug);
}

}  // extern "C"
