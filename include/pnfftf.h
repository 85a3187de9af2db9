/*
 * pnfftf.h -- the single-precision instantiation pnfftf_* of the PNFFT API.
 *
 * The reference declares one API per precision from the macro
 * PNFFT_DEFINE_API (api/pnfft.h:51-275) and expands it for float at
 * api/pnfft.h:287 (R = float, C = pnfftf_complex).  These are the same
 * functions, names and argument meanings with float arrays.  Timers stay
 * double and check_init_parameters takes a double x_max, as in the reference.
 *
 * Implementation: a layer over the double library.  The caller's float
 * arrays are kept; each pnfftf_trafo / pnfftf_adj converts them through
 * double staging arrays (page-locked) and runs the plan in the FP32-mixed
 * precision of the GPU path (pnfft_gb300_set_precision), or in FP64 when the
 * window overflows FP32.  Included by pnfft.h; may also be included after it.
 */
#ifndef PNFFTF_H
#define PNFFTF_H 1

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if !defined(__cplusplus) && defined(_Complex_I)
typedef float _Complex pnfftf_complex;
#else
typedef float pnfftf_complex[2];
#endif

typedef struct pnfftf_plan_s *pnfftf_plan;
typedef struct pnfftf_nodes_s *pnfftf_nodes;

int pnfftf_create_procmesh_2d(MPI_Comm comm, int np0, int np1, MPI_Comm *comm_cart_2d);
int pnfftf_create_procmesh(int rnk, MPI_Comm comm, const int *np, MPI_Comm *comm_cart);

void pnfftf_local_size_3d(const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                          ptrdiff_t *local_N_start, float *lower_border, float *upper_border);
void pnfftf_local_size_3d_c2r(const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                              ptrdiff_t *local_N_start, float *lower_border, float *upper_border);
void pnfftf_local_size_adv(int d, const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                           ptrdiff_t *local_N_start, float *lower_border, float *upper_border);
void pnfftf_local_size_adv_c2r(int d, const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags,
                               ptrdiff_t *local_N, ptrdiff_t *local_N_start, float *lower_border,
                               float *upper_border);
void pnfftf_local_size_guru(int d, const ptrdiff_t *N, const ptrdiff_t *n, const float *x_max, int m,
                            MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N, ptrdiff_t *local_N_start,
                            float *lower_border, float *upper_border);
void pnfftf_local_size_guru_c2r(int d, const ptrdiff_t *N, const ptrdiff_t *n, const float *x_max, int m,
                                MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                                ptrdiff_t *local_N_start, float *lower_border, float *upper_border);

pnfftf_plan pnfftf_init_3d(const ptrdiff_t *N, MPI_Comm comm_cart);
pnfftf_plan pnfftf_init_3d_c2r(const ptrdiff_t *N, MPI_Comm comm_cart);
pnfftf_plan pnfftf_init_adv(int d, const ptrdiff_t *N, unsigned pnfft_flags, unsigned pfft_flags,
                            MPI_Comm comm_cart);
pnfftf_plan pnfftf_init_adv_c2r(int d, const ptrdiff_t *N, unsigned pnfft_flags, unsigned pfft_flags,
                                MPI_Comm comm_cart);
pnfftf_plan pnfftf_init_guru(int d, const ptrdiff_t *N, const ptrdiff_t *n, const float *x_max, int m,
                             unsigned pnfft_flags, unsigned pfft_flags, MPI_Comm comm_cart);
pnfftf_plan pnfftf_init_guru_c2r(int d, const ptrdiff_t *N, const ptrdiff_t *n, const float *x_max, int m,
                                 unsigned pnfft_flags, unsigned pfft_flags, MPI_Comm comm_cart);

pnfftf_nodes pnfftf_init_nodes(ptrdiff_t local_M, unsigned malloc_flags);
void pnfftf_free_nodes(pnfftf_nodes nodes, unsigned pnfft_finalize_flags);
void pnfftf_precompute_psi(pnfftf_plan ths, pnfftf_nodes nodes, unsigned precompute_flags);

void pnfftf_set_f(pnfftf_complex *f, pnfftf_nodes nodes);
void pnfftf_set_grad_f(pnfftf_complex *grad_f, pnfftf_nodes nodes);
void pnfftf_set_hessian_f(pnfftf_complex *hessian_f, pnfftf_nodes nodes);
void pnfftf_set_f_real(float *f, pnfftf_nodes nodes);
void pnfftf_set_grad_f_real(float *grad_f, pnfftf_nodes nodes);
void pnfftf_set_hessian_f_real(float *hessian_f, pnfftf_nodes nodes);
void pnfftf_set_x(float *x, pnfftf_nodes nodes);
void pnfftf_set_f_hat(pnfftf_complex *f_hat, pnfftf_plan ths);
void pnfftf_set_f_hat_real(float *f_hat, pnfftf_plan ths);
void pnfftf_set_b(float b0, float b1, float b2, pnfftf_plan ths);

pnfftf_complex *pnfftf_get_f(const pnfftf_nodes nodes);
pnfftf_complex *pnfftf_get_grad_f(const pnfftf_nodes nodes);
pnfftf_complex *pnfftf_get_hessian_f(const pnfftf_nodes nodes);
float *pnfftf_get_f_real(const pnfftf_nodes nodes);
float *pnfftf_get_grad_f_real(const pnfftf_nodes nodes);
float *pnfftf_get_hessian_f_real(const pnfftf_nodes nodes);
float *pnfftf_get_x(const pnfftf_nodes nodes);
pnfftf_complex *pnfftf_get_f_hat(const pnfftf_plan ths);
float *pnfftf_get_f_hat_real(const pnfftf_plan ths);
int pnfftf_get_d(const pnfftf_plan ths);
int pnfftf_get_m(const pnfftf_plan ths);
void pnfftf_get_x_max(const pnfftf_plan ths, float *x_max);
void pnfftf_get_N(const pnfftf_plan ths, ptrdiff_t *N);
void pnfftf_get_n(const pnfftf_plan ths, ptrdiff_t *n);
unsigned pnfftf_get_pnfft_flags(const pnfftf_plan ths);
unsigned pnfftf_get_pfft_flags(const pnfftf_plan ths);
void pnfftf_get_b(const pnfftf_plan ths, float *b0, float *b1, float *b2);

void pnfftf_finalize(pnfftf_plan ths, unsigned pnfft_finalize_flags);
void pnfftf_trafo(pnfftf_plan ths, pnfftf_nodes nodes, unsigned compute_flags);
void pnfftf_adj(pnfftf_plan ths, pnfftf_nodes nodes, unsigned compute_flags);

void pnfftf_init(void);
void pnfftf_cleanup(void);
void *pnfftf_malloc(size_t n);
float *pnfftf_alloc_real(size_t n);
pnfftf_complex *pnfftf_alloc_complex(size_t n);
void pnfftf_free(void *p);

void pnfftf_init_f_hat_3d(const ptrdiff_t *N, const ptrdiff_t *local_N, const ptrdiff_t *local_N_start,
                          unsigned pnfft_flags, pnfftf_complex *data);
void pnfftf_init_f(ptrdiff_t local_M, pnfftf_complex *data);
void pnfftf_init_x_3d(const float *lo, const float *up, ptrdiff_t loc_M, float *x);
void pnfftf_init_x_3d_adv(const float *lo, const float *up, const float *x_max, ptrdiff_t loc_M, float *x);

void pnfftf_zero_f_hat(pnfftf_plan ths);
float pnfftf_inv_phi_hat(const pnfftf_plan ths, int dim, ptrdiff_t k);
float pnfftf_phi_hat(const pnfftf_plan ths, int dim, ptrdiff_t k);
float pnfftf_psi(const pnfftf_plan ths, int dim, float x);
float pnfftf_dpsi(const pnfftf_plan ths, int dim, float x);
float pnfftf_ddpsi(const pnfftf_plan ths, int dim, float x);

void pnfftf_vpr_complex(pnfftf_complex *data, ptrdiff_t N, const char *name, MPI_Comm comm);
void pnfftf_vpr_real(float *data, ptrdiff_t N, const char *name, MPI_Comm comm);
void pnfftf_apr_complex_3d(pnfftf_complex *data, ptrdiff_t *local_N, ptrdiff_t *local_N_start,
                           unsigned pnfft_flags, const char *name, MPI_Comm comm);
void pnfftf_apr_real_3d(float *data, ptrdiff_t *local_N, ptrdiff_t *local_N_start, unsigned pnfft_flags,
                        const char *name, MPI_Comm comm);

double *pnfftf_get_timer_trafo(pnfftf_plan ths);
double *pnfftf_get_timer_adj(pnfftf_plan ths);
void pnfftf_timer_average(double *timer);
double *pnfftf_timer_copy(const double *orig);
double *pnfftf_timer_reduce_max(MPI_Comm comm, double *timer);
double *pnfftf_timer_add(const double *sum1, const double *sum2);
void pnfftf_timer_free(double *ths);
void pnfftf_reset_timer(pnfftf_plan ths);
void pnfftf_print_average_timer(const pnfftf_plan ths, MPI_Comm comm);
void pnfftf_print_average_timer_adv(const pnfftf_plan ths, MPI_Comm comm);
void pnfftf_write_average_timer(const pnfftf_plan ths, const char *name, MPI_Comm comm);
void pnfftf_write_average_timer_adv(const pnfftf_plan ths, const char *name, MPI_Comm comm);

void pnfftf_get_args(int argc, char **argv, const char *name, int neededArgs, unsigned type, void *parameter);
void pnfftf_check_init_parameters(int argc, char **argv, ptrdiff_t *N, ptrdiff_t *n, ptrdiff_t *M, int *m,
                                  unsigned *pnfft_flags, unsigned *compute_flags, double *x_max, int *np,
                                  int *compare_direct, int *debug);

/* The double plan under a float plan (for the pnfft_gb300_* extensions:
 * precision, streams, device arrays).  No counterpart in the reference. */
pnfft_plan pnfftf_gb300_double_plan(pnfftf_plan ths);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* PNFFTF_H */
