/*
 * pnfft.h -- drop-in C interface of libpnfft_gb300 (double precision).
 *
 * Declares the same entry points, argument meanings and flag values as the
 * reference's api/pnfft.h (mpip/pnfft 1.0.7-alpha), whose declarations are
 * generated by the PNFFT_DEFINE_API macro at api/pnfft.h:51-275 and
 * instantiated for double at api/pnfft.h:286.  A plan on a one-process
 * communicator (1x1x1 process mesh) runs on one NVIDIA GB300 GPU; host
 * arrays are copied to and from the device inside each call.
 *
 * Each declaration below names the reference prototype (api/pnfft.h line)
 * and the reference implementation it replaces.
 *
 * MPI and PFFT are not needed: unless PNFFT_GB300_USE_MPI is defined before
 * this header is included, a single-rank stand-in for the few MPI names that
 * appear in the interface is provided (MPI_Comm is an int handle; only
 * MPI_COMM_WORLD and communicators returned by pnfft_create_procmesh* are
 * meaningful).  The PFFT planner flags accepted by pnfft_init_* are defined
 * here as well; they are stored and returned by pnfft_get_pfft_flags.
 */
#ifndef PNFFT_H
#define PNFFT_H 1

#include <stddef.h>
#include <math.h>

#ifdef PNFFT_GB300_USE_MPI
#include <mpi.h>
#else
#ifndef PNFFT_GB300_MPI_STUB
#define PNFFT_GB300_MPI_STUB 1
typedef int MPI_Comm;
#define MPI_COMM_WORLD ((MPI_Comm)0x44000000)
#define MPI_COMM_NULL ((MPI_Comm)0x04000000)
#endif
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* complex type: C99 double _Complex when <complex.h> was included before this
 * header (as the reference's own sources do), else two doubles (re, im). */
#if !defined(__cplusplus) && defined(_Complex_I)
typedef double _Complex pnfft_complex;
#else
typedef double pnfft_complex[2];
#endif

/* PFFT planner flags passed through pnfft_init_adv/guru (api/api-guru.c:168-190) */
#ifndef PFFT_ESTIMATE
#define PFFT_MEASURE (0U)
#define PFFT_ESTIMATE (1U << 0)
#define PFFT_PATIENT (1U << 1)
#define PFFT_EXHAUSTIVE (1U << 2)
#define PFFT_NO_TUNE (0U)
#define PFFT_TUNE (1U << 3)
#define PFFT_PRESERVE_INPUT (1U << 4)
#define PFFT_DESTROY_INPUT (1U << 5)
#define PFFT_BUFFERED_INPLACE (1U << 6)
#define PFFT_INT 1
#define PFFT_PTRDIFF_T 2
#define PFFT_FLOAT 3
#define PFFT_DOUBLE 4
#define PFFT_LDOUBLE 5
#define PFFT_UNSIGNED 6
#endif

typedef struct pnfft_plan_s *pnfft_plan;
typedef struct pnfft_nodes_s *pnfft_nodes;

/* ---- process mesh (api/pnfft.h:56-59; util/util.c:24-42) ------------------ */
/* Only meshes of total size 1 are accepted; returns 0 on success, 1 otherwise. */
int pnfft_create_procmesh_2d(MPI_Comm comm, int np0, int np1, MPI_Comm *comm_cart_2d);
int pnfft_create_procmesh(int rnk, MPI_Comm comm, const int *np, MPI_Comm *comm_cart);

/* ---- local sizes (api/pnfft.h:61-90; api/api-basic.c:36-63, api-adv.c:90-129,
 *      api-guru.c:42-107) --------------------------------------------------- */
void pnfft_local_size_3d(const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                         ptrdiff_t *local_N_start, double *lower_border, double *upper_border);
void pnfft_local_size_3d_c2r(const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                             ptrdiff_t *local_N_start, double *lower_border, double *upper_border);
void pnfft_local_size_adv(int d, const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                          ptrdiff_t *local_N_start, double *lower_border, double *upper_border);
void pnfft_local_size_adv_c2r(int d, const ptrdiff_t *N, MPI_Comm comm_cart, unsigned pnfft_flags,
                              ptrdiff_t *local_N, ptrdiff_t *local_N_start, double *lower_border,
                              double *upper_border);
void pnfft_local_size_guru(int d, const ptrdiff_t *N, const ptrdiff_t *n, const double *x_max, int m,
                           MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N, ptrdiff_t *local_N_start,
                           double *lower_border, double *upper_border);
void pnfft_local_size_guru_c2r(int d, const ptrdiff_t *N, const ptrdiff_t *n, const double *x_max, int m,
                               MPI_Comm comm_cart, unsigned pnfft_flags, ptrdiff_t *local_N,
                               ptrdiff_t *local_N_start, double *lower_border, double *upper_border);

/* ---- plan creation (api/pnfft.h:92-113; api-basic.c:66-97, api-adv.c:132-169,
 *      api-guru.c:64-164, kernel/ndft-parallel.c:869-1140) --------------------
 * Return NULL on error (d != 3, a mesh larger than 1, invalid sizes); the
 * reason is available from pnfft_gb300_last_error().  No GPU work happens
 * here: device buffers and cuFFT plans are created by the first transform. */
pnfft_plan pnfft_init_3d(const ptrdiff_t *N, MPI_Comm comm_cart);
pnfft_plan pnfft_init_3d_c2r(const ptrdiff_t *N, MPI_Comm comm_cart);
pnfft_plan pnfft_init_adv(int d, const ptrdiff_t *N, unsigned pnfft_flags, unsigned pfft_flags, MPI_Comm comm_cart);
pnfft_plan pnfft_init_adv_c2r(int d, const ptrdiff_t *N, unsigned pnfft_flags, unsigned pfft_flags,
                              MPI_Comm comm_cart);
pnfft_plan pnfft_init_guru(int d, const ptrdiff_t *N, const ptrdiff_t *n, const double *x_max, int m,
                           unsigned pnfft_flags, unsigned pfft_flags, MPI_Comm comm_cart);
pnfft_plan pnfft_init_guru_c2r(int d, const ptrdiff_t *N, const ptrdiff_t *n, const double *x_max, int m,
                               unsigned pnfft_flags, unsigned pfft_flags, MPI_Comm comm_cart);

/* ---- nodes (api/pnfft.h:115-122; api-basic.c:380-447, ndft-parallel.c:1144-1370) */
pnfft_nodes pnfft_init_nodes(ptrdiff_t local_M, unsigned malloc_flags);
void pnfft_free_nodes(pnfft_nodes nodes, unsigned pnfft_finalize_flags);
void pnfft_precompute_psi(pnfft_plan ths, pnfft_nodes nodes, unsigned precompute_flags);

/* ---- setters / getters (api/pnfft.h:124-181; api-basic.c:457-661) -------- */
void pnfft_set_f(pnfft_complex *f, pnfft_nodes nodes);
void pnfft_set_grad_f(pnfft_complex *grad_f, pnfft_nodes nodes);
void pnfft_set_hessian_f(pnfft_complex *hessian_f, pnfft_nodes nodes);
void pnfft_set_f_real(double *f, pnfft_nodes nodes);
void pnfft_set_grad_f_real(double *grad_f, pnfft_nodes nodes);
void pnfft_set_hessian_f_real(double *hessian_f, pnfft_nodes nodes);
void pnfft_set_x(double *x, pnfft_nodes nodes);
void pnfft_set_f_hat(pnfft_complex *f_hat, pnfft_plan ths);
void pnfft_set_f_hat_real(double *f_hat, pnfft_plan ths);
void pnfft_set_b(double b0, double b1, double b2, pnfft_plan ths);
pnfft_complex *pnfft_get_f(const pnfft_nodes nodes);
pnfft_complex *pnfft_get_grad_f(const pnfft_nodes nodes);
pnfft_complex *pnfft_get_hessian_f(const pnfft_nodes nodes);
double *pnfft_get_f_real(const pnfft_nodes nodes);
double *pnfft_get_grad_f_real(const pnfft_nodes nodes);
double *pnfft_get_hessian_f_real(const pnfft_nodes nodes);
double *pnfft_get_x(const pnfft_nodes nodes);
pnfft_complex *pnfft_get_f_hat(const pnfft_plan ths);
double *pnfft_get_f_hat_real(const pnfft_plan ths);
int pnfft_get_d(const pnfft_plan ths);
int pnfft_get_m(const pnfft_plan ths);
void pnfft_get_x_max(const pnfft_plan ths, double *x_max);
void pnfft_get_N(const pnfft_plan ths, ptrdiff_t *N);
void pnfft_get_n(const pnfft_plan ths, ptrdiff_t *n);
unsigned pnfft_get_pnfft_flags(const pnfft_plan ths);
unsigned pnfft_get_pfft_flags(const pnfft_plan ths);
void pnfft_get_b(const pnfft_plan ths, double *b0, double *b1, double *b2);

/* ---- transforms (api/pnfft.h:183-189; api-basic.c:170-378) ----------------
 * f = B F D f_hat (trafo) and f_hat = D^T F^H B^T f (adj) on the GPU.  Outputs
 * are overwritten unless PNFFT_COMPUTE_ACCUMULATED; a NULL plan, or NULL
 * nodes without PNFFT_OMIT_CONV, returns without work (api-basic.c:205-206). */
void pnfft_finalize(pnfft_plan ths, unsigned pnfft_finalize_flags);
void pnfft_trafo(pnfft_plan ths, pnfft_nodes nodes, unsigned compute_flags);
void pnfft_adj(pnfft_plan ths, pnfft_nodes nodes, unsigned compute_flags);

/* ---- library set-up (api/pnfft.h:191-194; api-basic.c:27-34) ------------- */
void pnfft_init(void);
void pnfft_cleanup(void);

/* ---- memory (api/pnfft.h:196-199; kernel/malloc.c) -----------------------
 * Returns page-locked host memory when a GPU is present (faster copies),
 * else aligned heap memory; release with pnfft_free. */
void *pnfft_malloc(size_t n);
double *pnfft_alloc_real(size_t n);
pnfft_complex *pnfft_alloc_complex(size_t n);
void pnfft_free(void *p);

/* ---- test-input generators (api/pnfft.h:201-213; api-basic.c:663-702,
 *      api-adv.c:35-86) ------------------------------------------------------ */
void pnfft_init_f_hat_3d(const ptrdiff_t *N, const ptrdiff_t *local_N, const ptrdiff_t *local_N_start,
                         unsigned pnfft_flags, pnfft_complex *data);
void pnfft_init_f(ptrdiff_t local_M, pnfft_complex *data);
void pnfft_init_x_3d(const double *lo, const double *up, ptrdiff_t loc_M, double *x);
void pnfft_init_x_3d_adv(const double *lo, const double *up, const double *x_max, ptrdiff_t loc_M, double *x);

void pnfft_zero_f_hat(pnfft_plan ths);

/* ---- window functions (api/pnfft.h:218-227; matrix_D.c:191-225,
 *      ndft-parallel.c:2288-2334), evaluated on the host in FP64 ------------- */
double pnfft_inv_phi_hat(const pnfft_plan ths, int dim, ptrdiff_t k);
double pnfft_phi_hat(const pnfft_plan ths, int dim, ptrdiff_t k);
double pnfft_psi(const pnfft_plan ths, int dim, double x);
double pnfft_dpsi(const pnfft_plan ths, int dim, double x);
double pnfft_ddpsi(const pnfft_plan ths, int dim, double x);

/* ---- printing (api/pnfft.h:229-238; api-basic.c:705-818) ------------------ */
void pnfft_vpr_complex(pnfft_complex *data, ptrdiff_t N, const char *name, MPI_Comm comm);
void pnfft_vpr_real(double *data, ptrdiff_t N, const char *name, MPI_Comm comm);
void pnfft_apr_complex_3d(pnfft_complex *data, ptrdiff_t *local_N, ptrdiff_t *local_N_start, unsigned pnfft_flags,
                          const char *name, MPI_Comm comm);
void pnfft_apr_real_3d(double *data, ptrdiff_t *local_N, ptrdiff_t *local_N_start, unsigned pnfft_flags,
                       const char *name, MPI_Comm comm);

/* ---- timers (api/pnfft.h:240-264; kernel/timer.c) ------------------------
 * Stage times are taken with CUDA events on the plan's stream, in seconds. */
double *pnfft_get_timer_trafo(pnfft_plan ths);
double *pnfft_get_timer_adj(pnfft_plan ths);
void pnfft_timer_average(double *timer);
double *pnfft_timer_copy(const double *orig);
double *pnfft_timer_reduce_max(MPI_Comm comm, double *timer);
double *pnfft_timer_add(const double *sum1, const double *sum2);
void pnfft_timer_free(double *ths);
void pnfft_reset_timer(pnfft_plan ths);
void pnfft_print_average_timer(const pnfft_plan ths, MPI_Comm comm);
void pnfft_print_average_timer_adv(const pnfft_plan ths, MPI_Comm comm);
void pnfft_write_average_timer(const pnfft_plan ths, const char *name, MPI_Comm comm);
void pnfft_write_average_timer_adv(const pnfft_plan ths, const char *name, MPI_Comm comm);

/* ---- command line (api/pnfft.h:266-275; util/getargs.c, api-basic.c:820-953) */
void pnfft_get_args(int argc, char **argv, const char *name, int neededArgs, unsigned type, void *parameter);
void pnfft_check_init_parameters(int argc, char **argv, ptrdiff_t *N, ptrdiff_t *n, ptrdiff_t *M, int *m,
                                 unsigned *pnfft_flags, unsigned *compute_flags, double *x_max, int *np,
                                 int *compare_direct, int *debug);

#ifndef PNFFT_PI
#define PNFFT_PI 3.14159265358979323846
#endif

/* ---- plan flags (api/pnfft.h:302-334) ------------------------------------ */
#define PNFFT_PRE_PHI_HAT (1U << 0)
#define PNFFT_PRE_PHI_HUT PNFFT_PRE_PHI_HAT
#define PNFFT_FAST_GAUSSIAN (1U << 1)
#define PNFFT_PRE_CONST_PSI (1U << 2)
#define PNFFT_PRE_LIN_PSI (1U << 3)
#define PNFFT_PRE_QUAD_PSI (1U << 4)
#define PNFFT_PRE_CUB_PSI (1U << 5)
#define PNFFT_PRE_INTPOL_PSI (PNFFT_PRE_CONST_PSI | PNFFT_PRE_LIN_PSI | PNFFT_PRE_QUAD_PSI | PNFFT_PRE_CUB_PSI)
#define PNFFT_MALLOC_F_HAT (1U << 6)
#define PNFFT_FFT_OUT_OF_PLACE (0U)
#define PNFFT_FFT_IN_PLACE (1U << 7)
#define PNFFT_INTERLACED (1U << 8)
#define PNFFT_SHIFTED_F_HAT (1U << 9)
#define PNFFT_SHIFTED_X (1U << 10)
#define PNFFT_TRANSPOSED_NONE (0U)
#define PNFFT_TRANSPOSED_F_HAT (1U << 11)
#define PNFFT_DIFF_AD (0U)
#define PNFFT_DIFF_IK (1U << 12)
#define PNFFT_WINDOW_KAISER_BESSEL (0U)
#define PNFFT_WINDOW_GAUSSIAN (1U << 13)
#define PNFFT_WINDOW_BSPLINE (1U << 14)
#define PNFFT_WINDOW_SINC_POWER (1U << 15)
#define PNFFT_WINDOW_BESSEL_I0 (1U << 16)
#define PNFFT_USE_FK_GAUSSIAN_T (1U << 17)
#define PNFFT_WINDOW_GAUSSIAN_T (PNFFT_USE_FK_GAUSSIAN_T | PNFFT_WINDOW_GAUSSIAN)
#define PNFFT_SORT_NODES (1U << 18)

/* plan finalization (api/pnfft.h:340) */
#define PNFFT_FREE_F_HAT PNFFT_MALLOC_F_HAT

/* node initialization / finalization (api/pnfft.h:345-377) */
#define PNFFT_MALLOC_NONE (0U)
#define PNFFT_MALLOC_X (1U << 0)
#define PNFFT_MALLOC_F (1U << 1)
#define PNFFT_MALLOC_GRAD_F (1U << 2)
#define PNFFT_MALLOC_HESSIAN_F (1U << 3)
#define PNFFT_MALLOC_ALL (PNFFT_MALLOC_X | PNFFT_MALLOC_F | PNFFT_MALLOC_GRAD_F | PNFFT_MALLOC_HESSIAN_F)
#define PNFFT_REAL_F (1U << 4)
#define PNFFT_FREE_NONE (0U)
#define PNFFT_FREE_X PNFFT_MALLOC_X
#define PNFFT_FREE_F PNFFT_MALLOC_F
#define PNFFT_FREE_GRAD_F PNFFT_MALLOC_GRAD_F
#define PNFFT_FREE_HESSIAN_F PNFFT_MALLOC_HESSIAN_F
#define PNFFT_FREE_ALL PNFFT_MALLOC_ALL

/* window precomputation (api/pnfft.h:359-364) */
#define PNFFT_PRE_TENSOR (0U)
#define PNFFT_PRE_FULL (1U << 0)
#define PNFFT_PRE_PSI (1U << 1)
#define PNFFT_PRE_GRAD_PSI (1U << 2)
#define PNFFT_PRE_HESSIAN_PSI (1U << 3)

/* execution (api/pnfft.h:383-390) */
#define PNFFT_COMPUTE_F (1U << 0)
#define PNFFT_COMPUTE_GRAD_F (1U << 1)
#define PNFFT_COMPUTE_HESSIAN_F (1U << 2)
#define PNFFT_COMPUTE_DIRECT (1U << 3)
#define PNFFT_COMPUTE_ACCUMULATED (1U << 4)
#define PNFFT_OMIT_DECONV (1U << 5)
#define PNFFT_OMIT_FFT (1U << 6)
#define PNFFT_OMIT_CONV (1U << 7)

/* command-line argument types (api/pnfft.h:396-401) */
#define PNFFT_INT PFFT_INT
#define PNFFT_PTRDIFF_T PFFT_PTRDIFF_T
#define PNFFT_FLOAT PFFT_FLOAT
#define PNFFT_DOUBLE PFFT_DOUBLE
#define PNFFT_LDOUBLE PFFT_LDOUBLE
#define PNFFT_UNSIGNED PFFT_UNSIGNED

/* timer indices (api/pnfft.h:407-418) */
#define PNFFT_TIMER_ITER (0)
#define PNFFT_TIMER_WHOLE (1)
#define PNFFT_TIMER_LOOP_B (2)
#define PNFFT_TIMER_SORT_NODES (3)
#define PNFFT_TIMER_GCELLS (4)
#define PNFFT_TIMER_MATRIX_B (5)
#define PNFFT_TIMER_MATRIX_F (6)
#define PNFFT_TIMER_MATRIX_D (7)
#define PNFFT_TIMER_SHIFT_INPUT (8)
#define PNFFT_TIMER_SHIFT_OUTPUT (9)
#define PNFFT_TIMER_LENGTH (10)

#ifdef __cplusplus
} /* extern "C" */
#endif

#include "pnfft_gb300.h"
#include "pnfftf.h"

#endif /* PNFFT_H */
