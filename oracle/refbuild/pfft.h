/* pfft.h -- single-process stand-in for the PFFT interface that the
 * reference PNFFT sources use (TEST INFRASTRUCTURE: only for building the
 * reference's own C code into oracle/_ref/ to pin the oracle).
 *
 * It follows PFFT's documented semantics for one process and complex data:
 *  - local sizes: the whole arrays, starting at -N/2 (PFFT_SHIFTED_IN) and
 *    -no/2 (PFFT_SHIFTED_OUT);
 *  - pruned, shifted c2c transforms: the forward plan maps the input block
 *    k in [-ni/2, ni/2) to the outputs l in [-no/2, no/2),
 *    out[l] = sum_k in[k] exp(sign 2 pi i k.l / n), with no normalisation;
 *  - ghost cells: exchange turns the contiguous no-block into the block with
 *    gc_below / gc_above periodic copies on each side, reduce adds the ghost
 *    values back onto the periodic interior and returns the contiguous block.
 * Only what a 1x1x1 c2c plan without PFFT_TRANSPOSED_* touches is provided;
 * the c2r/r2c entry points and transposed layouts abort. */
#ifndef ORACLE_REFBUILD_PFFT_H
#define ORACLE_REFBUILD_PFFT_H
#include <complex.h>
#include <stddef.h>
#include <stdio.h>

#include <mpi.h>

#define PFFT_MANGLE_DOUBLE(name) pfft_##name
#define PFFT_MANGLE_FLOAT(name) pfftf_##name
#define PFFT_MANGLE_LONG_DOUBLE(name) pfftl_##name
#define FFTW_MANGLE_DOUBLE(name) fftw_##name
#define FFTW_MANGLE_FLOAT(name) fftwf_##name
#define FFTW_MANGLE_LONG_DOUBLE(name) fftwl_##name

typedef double _Complex pfft_complex;
typedef float _Complex pfftf_complex;
typedef long double _Complex pfftl_complex;
typedef struct pfft_plan_s *pfft_plan;
typedef struct pfft_gcplan_s *pfft_gcplan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define PFFT_FORWARD (-1)
#define PFFT_BACKWARD (+1)
#define PFFT_DEFAULT_BLOCKS ((const ptrdiff_t *)0)

#define PFFT_TRANSPOSED_NONE (0U)
#define PFFT_TRANSPOSED_IN (1U << 0)
#define PFFT_TRANSPOSED_OUT (1U << 1)
#define PFFT_SHIFTED_IN (1U << 2)
#define PFFT_SHIFTED_OUT (1U << 3)
#define PFFT_MEASURE (0U)
#define PFFT_ESTIMATE (1U << 4)
#define PFFT_PATIENT (1U << 5)
#define PFFT_EXHAUSTIVE (1U << 6)
#define PFFT_NO_TUNE (0U)
#define PFFT_TUNE (1U << 7)
#define PFFT_PRESERVE_INPUT (1U << 8)
#define PFFT_DESTROY_INPUT (1U << 9)

/* argument types of pfft_get_args */
#define PFFT_INT 1
#define PFFT_PTRDIFF_T 2
#define PFFT_FLOAT 3
#define PFFT_DOUBLE 4
#define PFFT_LDOUBLE 5
#define PFFT_UNSIGNED 6

void pfft_init(void);
void pfft_cleanup(void);
int pfft_create_procmesh(int rnk, MPI_Comm comm, const int *np, MPI_Comm *comm_cart);
int pfft_create_procmesh_2d(MPI_Comm comm, int np0, int np1, MPI_Comm *comm_cart_2d);

ptrdiff_t pfft_prod_INT(int d, const ptrdiff_t *vec);
ptrdiff_t pfft_sum_INT(int d, const ptrdiff_t *vec);
int pfft_equal_INT(int d, const ptrdiff_t *vec1, const ptrdiff_t *vec2);
void pfft_vcopy_INT(int d, const ptrdiff_t *vec1, ptrdiff_t *vec2);
void pfft_vadd_INT(int d, const ptrdiff_t *vec1, const ptrdiff_t *vec2, ptrdiff_t *sum);
void pfft_vsub_INT(int d, const ptrdiff_t *vec1, const ptrdiff_t *vec2, ptrdiff_t *sub);

ptrdiff_t pfft_local_size_many_dft(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                                   ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock,
                                   MPI_Comm comm_cart, unsigned pfft_flags, ptrdiff_t *local_ni,
                                   ptrdiff_t *local_i_start, ptrdiff_t *local_no, ptrdiff_t *local_o_start);
ptrdiff_t pfft_local_size_many_dft_c2r(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                                       ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock,
                                       MPI_Comm comm_cart, unsigned pfft_flags, ptrdiff_t *local_ni,
                                       ptrdiff_t *local_i_start, ptrdiff_t *local_no, ptrdiff_t *local_o_start);
ptrdiff_t pfft_local_size_many_dft_r2c(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                                       ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock,
                                       MPI_Comm comm_cart, unsigned pfft_flags, ptrdiff_t *local_ni,
                                       ptrdiff_t *local_i_start, ptrdiff_t *local_no, ptrdiff_t *local_o_start);
void pfft_local_block_many_dft(int rnk, const ptrdiff_t *ni, const ptrdiff_t *no, const ptrdiff_t *iblock,
                               const ptrdiff_t *oblock, MPI_Comm comm_cart, int pid, unsigned pfft_flags,
                               ptrdiff_t *local_ni, ptrdiff_t *local_i_start, ptrdiff_t *local_no,
                               ptrdiff_t *local_o_start);
void pfft_local_block_many_dft_c2r(int rnk, const ptrdiff_t *ni, const ptrdiff_t *no, const ptrdiff_t *iblock,
                                   const ptrdiff_t *oblock, MPI_Comm comm_cart, int pid, unsigned pfft_flags,
                                   ptrdiff_t *local_ni, ptrdiff_t *local_i_start, ptrdiff_t *local_no,
                                   ptrdiff_t *local_o_start);
pfft_plan pfft_plan_many_dft(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                             ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock, pfft_complex *in,
                             pfft_complex *out, MPI_Comm comm_cart, int sign, unsigned pfft_flags);
pfft_plan pfft_plan_many_dft_c2r(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                                 ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock,
                                 pfft_complex *in, double *out, MPI_Comm comm_cart, int sign, unsigned pfft_flags);
pfft_plan pfft_plan_many_dft_r2c(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                                 ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock, double *in,
                                 pfft_complex *out, MPI_Comm comm_cart, int sign, unsigned pfft_flags);
void pfft_execute(const pfft_plan plan);
void pfft_destroy_plan(pfft_plan plan);

ptrdiff_t pfft_local_size_many_gc(int rnk, const ptrdiff_t *local_n, const ptrdiff_t *local_start,
                                  ptrdiff_t howmany, const ptrdiff_t *gc_below, const ptrdiff_t *gc_above,
                                  ptrdiff_t *local_ngc, ptrdiff_t *local_gc_start);
pfft_gcplan pfft_plan_many_cgc(int rnk, const ptrdiff_t *n, ptrdiff_t howmany, const ptrdiff_t *block,
                               const ptrdiff_t *gc_below, const ptrdiff_t *gc_above, pfft_complex *data,
                               MPI_Comm comm_cart, unsigned gc_flags);
pfft_gcplan pfft_plan_many_rgc(int rnk, const ptrdiff_t *n, ptrdiff_t howmany, const ptrdiff_t *block,
                               const ptrdiff_t *gc_below, const ptrdiff_t *gc_above, double *data,
                               MPI_Comm comm_cart, unsigned gc_flags);
void pfft_exchange(pfft_gcplan plan);
void pfft_reduce(pfft_gcplan plan);
void pfft_destroy_gcplan(pfft_gcplan plan);

void *pfft_malloc(size_t n);
double *pfft_alloc_real(size_t n);
pfft_complex *pfft_alloc_complex(size_t n);
void pfft_free(void *p);

void pfft_fprintf(MPI_Comm comm, FILE *stream, const char *format, ...);
void pfft_printf(MPI_Comm comm, const char *format, ...);
void pfft_init_input_complex_3d(const ptrdiff_t *n, const ptrdiff_t *local_n, const ptrdiff_t *local_start,
                                pfft_complex *data);
void pfft_apr_complex_3d(const pfft_complex *data, const ptrdiff_t *local_n, const ptrdiff_t *local_start,
                         const char *name, MPI_Comm comm);
void pfft_apr_real_3d(const double *data, const ptrdiff_t *local_n, const ptrdiff_t *local_start, const char *name,
                      MPI_Comm comm);
void pfft_get_args(int argc, char **argv, const char *name, int neededArgs, unsigned type, void *parameter);
#endif
