/*
 * shim.c -- single-process stand-ins for MPI, PFFT and two GSL functions,
 * against which the reference PNFFT C sources are compiled unmodified into
 * oracle/_ref/libpnfft_ref.so (build recipe: oracle/build_ref.py).
 *
 * TEST INFRASTRUCTURE ONLY.  The resulting library is the reference's own
 * trafo/adj code path on a 1x1x1 process mesh; the tests use it to pin the
 * oracle (oracle/pnfft_oracle.c) to the reference itself.  The F step is this
 * file's FP64 FFT, not FFTW, and the ghost-cell exchange/reduce are this
 * file's periodic copies; the semantics follow the comment in pfft.h.  Nothing
 * in the product links or loads it.
 */
#include <complex.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "gsl/gsl_sf_bessel.h"
#include "mpi.h"
#include "pfft.h"

static void die(const char *what) {
  fprintf(stderr, "oracle reference build: %s is not provided by the single-process stand-in\n", what);
  abort();
}

/* ------------------------------------------------------------------------- */
/* MPI: one rank                                                              */
/* ------------------------------------------------------------------------- */
static size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_CHAR: return 1;
    case MPI_INT: return sizeof(int);
    case MPI_UNSIGNED: return sizeof(unsigned);
    case MPI_LONG: return sizeof(long);
    case MPI_FLOAT: return sizeof(float);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_LONG_DOUBLE: return sizeof(long double);
    case MPI_LONG_LONG: return sizeof(long long);
    default: die("this MPI datatype");
  }
  return 0;
}
int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm *newcomm) { *newcomm = comm; return MPI_SUCCESS; }
int MPI_Comm_free(MPI_Comm *comm) { *comm = MPI_COMM_NULL; return MPI_SUCCESS; }
int MPI_Cartdim_get(MPI_Comm comm, int *ndims) { (void)comm; *ndims = 3; return MPI_SUCCESS; }
int MPI_Cart_get(MPI_Comm comm, int maxdims, int *dims, int *periods, int *coords) {
  (void)comm;
  for (int t = 0; t < maxdims; t++) {
    dims[t] = 1;
    periods[t] = 1;
    coords[t] = 0;
  }
  return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm comm) { (void)comm; return MPI_SUCCESS; }
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm) {
  (void)buf; (void)count; (void)type; (void)root; (void)comm;
  return MPI_SUCCESS;
}
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, int root,
               MPI_Comm comm) {
  (void)op; (void)root; (void)comm;
  if (sendbuf != recvbuf) memmove(recvbuf, sendbuf, (size_t)count * type_size(type));
  return MPI_SUCCESS;
}
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm) {
  return MPI_Reduce(sendbuf, recvbuf, count, type, op, 0, comm);
}
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ------------------------------------------------------------------------- */
/* GSL I0, I1: power series sum_k (x/2)^(2k+nu) / (k! (k+nu)!), all terms    */
/* positive, summed until they no longer change the sum                      */
/* ------------------------------------------------------------------------- */
static double bessel_series(int nu, double x) {
  const double h = 0.5 * fabs(x), q = h * h;
  double term = nu ? h : 1.0, sum = term;
  for (int k = 1; k < 2000; k++) {
    term *= q / ((double)k * (double)(k + nu));
    const double s = sum + term;
    if (s == sum) break;
    sum = s;
  }
  return (nu && x < 0) ? -sum : sum;
}
double gsl_sf_bessel_I0(double x) { return bessel_series(0, x); }
double gsl_sf_bessel_I1(double x) { return bessel_series(1, x); }

/* ------------------------------------------------------------------------- */
/* PFFT: utilities                                                           */
/* ------------------------------------------------------------------------- */
void pfft_init(void) {}
void pfft_cleanup(void) {}
int pfft_create_procmesh(int rnk, MPI_Comm comm, const int *np, MPI_Comm *comm_cart) {
  for (int t = 0; t < rnk; t++)
    if (np[t] != 1) return 1;
  *comm_cart = comm;
  return 0;
}
int pfft_create_procmesh_2d(MPI_Comm comm, int np0, int np1, MPI_Comm *comm_cart_2d) {
  if (np0 != 1 || np1 != 1) return 1;
  *comm_cart_2d = comm;
  return 0;
}
ptrdiff_t pfft_prod_INT(int d, const ptrdiff_t *vec) {
  ptrdiff_t p = 1;
  for (int t = 0; t < d; t++) p *= vec[t];
  return p;
}
ptrdiff_t pfft_sum_INT(int d, const ptrdiff_t *vec) {
  ptrdiff_t s = 0;
  for (int t = 0; t < d; t++) s += vec[t];
  return s;
}
int pfft_equal_INT(int d, const ptrdiff_t *vec1, const ptrdiff_t *vec2) {
  for (int t = 0; t < d; t++)
    if (vec1[t] != vec2[t]) return 0;
  return 1;
}
void pfft_vcopy_INT(int d, const ptrdiff_t *vec1, ptrdiff_t *vec2) {
  for (int t = 0; t < d; t++) vec2[t] = vec1[t];
}
void pfft_vadd_INT(int d, const ptrdiff_t *vec1, const ptrdiff_t *vec2, ptrdiff_t *sum) {
  for (int t = 0; t < d; t++) sum[t] = vec1[t] + vec2[t];
}
void pfft_vsub_INT(int d, const ptrdiff_t *vec1, const ptrdiff_t *vec2, ptrdiff_t *sub) {
  for (int t = 0; t < d; t++) sub[t] = vec1[t] - vec2[t];
}
void *pfft_malloc(size_t n) {
  void *p = NULL;
  if (posix_memalign(&p, 64, n ? n : 1)) return NULL;
  return p;
}
double *pfft_alloc_real(size_t n) { return (double *)pfft_malloc(sizeof(double) * n); }
pfft_complex *pfft_alloc_complex(size_t n) { return (pfft_complex *)pfft_malloc(sizeof(pfft_complex) * n); }
void pfft_free(void *p) { free(p); }
void pfft_fprintf(MPI_Comm comm, FILE *stream, const char *format, ...) {
  (void)comm;
  va_list ap;
  va_start(ap, format);
  vfprintf(stream, format, ap);
  va_end(ap);
}
void pfft_printf(MPI_Comm comm, const char *format, ...) {
  (void)comm;
  va_list ap;
  va_start(ap, format);
  vfprintf(stdout, format, ap);
  va_end(ap);
}
void pfft_init_input_complex_3d(const ptrdiff_t *n, const ptrdiff_t *local_n, const ptrdiff_t *local_start,
                                pfft_complex *data) {
  (void)n; (void)local_n; (void)local_start; (void)data;
  die("pfft_init_input_complex_3d");
}
void pfft_apr_complex_3d(const pfft_complex *data, const ptrdiff_t *local_n, const ptrdiff_t *local_start,
                         const char *name, MPI_Comm comm) {
  (void)data; (void)local_n; (void)local_start; (void)name; (void)comm;
}
void pfft_apr_real_3d(const double *data, const ptrdiff_t *local_n, const ptrdiff_t *local_start, const char *name,
                      MPI_Comm comm) {
  (void)data; (void)local_n; (void)local_start; (void)name; (void)comm;
}
void pfft_get_args(int argc, char **argv, const char *name, int neededArgs, unsigned type, void *parameter) {
  (void)argc; (void)argv; (void)name; (void)neededArgs; (void)type; (void)parameter;
}
void pfft_print_average_timer_adv(const pfft_plan plan, MPI_Comm comm) { (void)plan; (void)comm; }
void pfft_write_average_timer_adv(const pfft_plan plan, const char *name, MPI_Comm comm) {
  (void)plan; (void)name; (void)comm;
}
void pfft_print_average_gctimer_adv(const pfft_gcplan plan, MPI_Comm comm) { (void)plan; (void)comm; }
void pfft_write_average_gctimer_adv(const pfft_gcplan plan, const char *name, MPI_Comm comm) {
  (void)plan; (void)name; (void)comm;
}

/* ------------------------------------------------------------------------- */
/* PFFT: local sizes of a one-process mesh                                   */
/* ------------------------------------------------------------------------- */
static void whole_block(int rnk, const ptrdiff_t *nn, unsigned shifted, ptrdiff_t *local_n, ptrdiff_t *start) {
  for (int t = 0; t < rnk; t++) {
    local_n[t] = nn[t];
    start[t] = shifted ? -(nn[t] / 2) : 0;
  }
}
ptrdiff_t pfft_local_size_many_dft(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                                   ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock,
                                   MPI_Comm comm_cart, unsigned pfft_flags, ptrdiff_t *local_ni,
                                   ptrdiff_t *local_i_start, ptrdiff_t *local_no, ptrdiff_t *local_o_start) {
  (void)n; (void)iblock; (void)oblock; (void)comm_cart;
  if (pfft_flags & (PFFT_TRANSPOSED_IN | PFFT_TRANSPOSED_OUT)) die("the transposed layouts");
  whole_block(rnk, ni, pfft_flags & PFFT_SHIFTED_IN, local_ni, local_i_start);
  whole_block(rnk, no, pfft_flags & PFFT_SHIFTED_OUT, local_no, local_o_start);
  const ptrdiff_t a = pfft_prod_INT(rnk, ni), b = pfft_prod_INT(rnk, no);
  return howmany * (a > b ? a : b);
}
ptrdiff_t pfft_local_size_many_dft_c2r(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                                       ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock,
                                       MPI_Comm comm_cart, unsigned pfft_flags, ptrdiff_t *local_ni,
                                       ptrdiff_t *local_i_start, ptrdiff_t *local_no, ptrdiff_t *local_o_start) {
  (void)rnk; (void)n; (void)ni; (void)no; (void)howmany; (void)iblock; (void)oblock; (void)comm_cart;
  (void)pfft_flags; (void)local_ni; (void)local_i_start; (void)local_no; (void)local_o_start;
  die("the c2r transforms");
  return 0;
}
ptrdiff_t pfft_local_size_many_dft_r2c(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                                       ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock,
                                       MPI_Comm comm_cart, unsigned pfft_flags, ptrdiff_t *local_ni,
                                       ptrdiff_t *local_i_start, ptrdiff_t *local_no, ptrdiff_t *local_o_start) {
  return pfft_local_size_many_dft_c2r(rnk, n, ni, no, howmany, iblock, oblock, comm_cart, pfft_flags, local_ni,
                                      local_i_start, local_no, local_o_start);
}
void pfft_local_block_many_dft(int rnk, const ptrdiff_t *ni, const ptrdiff_t *no, const ptrdiff_t *iblock,
                               const ptrdiff_t *oblock, MPI_Comm comm_cart, int pid, unsigned pfft_flags,
                               ptrdiff_t *local_ni, ptrdiff_t *local_i_start, ptrdiff_t *local_no,
                               ptrdiff_t *local_o_start) {
  (void)iblock; (void)oblock; (void)comm_cart; (void)pid;
  if (pfft_flags & (PFFT_TRANSPOSED_IN | PFFT_TRANSPOSED_OUT)) die("the transposed layouts");
  whole_block(rnk, ni, pfft_flags & PFFT_SHIFTED_IN, local_ni, local_i_start);
  whole_block(rnk, no, pfft_flags & PFFT_SHIFTED_OUT, local_no, local_o_start);
}
void pfft_local_block_many_dft_c2r(int rnk, const ptrdiff_t *ni, const ptrdiff_t *no, const ptrdiff_t *iblock,
                                   const ptrdiff_t *oblock, MPI_Comm comm_cart, int pid, unsigned pfft_flags,
                                   ptrdiff_t *local_ni, ptrdiff_t *local_i_start, ptrdiff_t *local_no,
                                   ptrdiff_t *local_o_start) {
  (void)rnk; (void)ni; (void)no; (void)iblock; (void)oblock; (void)comm_cart; (void)pid; (void)pfft_flags;
  (void)local_ni; (void)local_i_start; (void)local_no; (void)local_o_start;
  die("the c2r transforms");
}

/* ------------------------------------------------------------------------- */
/* PFFT: pruned, shifted c2c transforms (FP64)                               */
/* ------------------------------------------------------------------------- */
struct pfft_plan_s {
  ptrdiff_t n[3], ni[3], no[3];
  pfft_complex *in, *out;
  int sign;
};

/* in-place 1-D DFT of length len at stride st, sign s: radix-2 for powers of
 * two, the direct sum with exact twiddle indices otherwise */
static void dft1(pfft_complex *a, ptrdiff_t len, ptrdiff_t st, int s, pfft_complex *tmp) {
  const double tw = (double)s * 2.0 * M_PI / (double)len;
  if ((len & (len - 1)) == 0) {
    for (ptrdiff_t i = 0; i < len; i++) tmp[i] = a[i * st];
    for (ptrdiff_t i = 1, j = 0; i < len; i++) { /* bit reversal */
      ptrdiff_t bit = len >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) {
        pfft_complex t = tmp[i];
        tmp[i] = tmp[j];
        tmp[j] = t;
      }
    }
    for (ptrdiff_t h = 1; h < len; h <<= 1)
      for (ptrdiff_t k = 0; k < h; k++) {
        const ptrdiff_t e = k * (len / (2 * h));
        const pfft_complex w = cos(tw * (double)e) + I * sin(tw * (double)e);
        for (ptrdiff_t i = k; i < len; i += 2 * h) {
          const pfft_complex u = tmp[i], v = tmp[i + h] * w;
          tmp[i] = u + v;
          tmp[i + h] = u - v;
        }
      }
  } else {
    for (ptrdiff_t l = 0; l < len; l++) {
      pfft_complex acc = 0;
      for (ptrdiff_t k = 0; k < len; k++) {
        const ptrdiff_t e = (k * l) % len;
        acc += a[k * st] * (cos(tw * (double)e) + I * sin(tw * (double)e));
      }
      tmp[l] = acc;
    }
  }
  for (ptrdiff_t i = 0; i < len; i++) a[i * st] = tmp[i];
}

static ptrdiff_t wrapn(ptrdiff_t i, ptrdiff_t n) {
  ptrdiff_t w = i % n;
  return w < 0 ? w + n : w;
}

pfft_plan pfft_plan_many_dft(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                             ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock, pfft_complex *in,
                             pfft_complex *out, MPI_Comm comm_cart, int sign, unsigned pfft_flags) {
  (void)iblock; (void)oblock; (void)comm_cart;
  if (rnk != 3 || howmany != 1) die("this transform rank or howmany");
  if (pfft_flags & (PFFT_TRANSPOSED_IN | PFFT_TRANSPOSED_OUT)) die("the transposed layouts");
  if (!(pfft_flags & PFFT_SHIFTED_IN) || !(pfft_flags & PFFT_SHIFTED_OUT)) die("unshifted transforms");
  struct pfft_plan_s *p = (struct pfft_plan_s *)calloc(1, sizeof(*p));
  for (int t = 0; t < 3; t++) {
    p->n[t] = n[t];
    p->ni[t] = ni[t];
    p->no[t] = no[t];
  }
  p->in = in;
  p->out = out;
  p->sign = sign;
  return p;
}
pfft_plan pfft_plan_many_dft_c2r(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                                 ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock,
                                 pfft_complex *in, double *out, MPI_Comm comm_cart, int sign, unsigned pfft_flags) {
  (void)rnk; (void)n; (void)ni; (void)no; (void)howmany; (void)iblock; (void)oblock; (void)in; (void)out;
  (void)comm_cart; (void)sign; (void)pfft_flags;
  die("the c2r transforms");
  return NULL;
}
pfft_plan pfft_plan_many_dft_r2c(int rnk, const ptrdiff_t *n, const ptrdiff_t *ni, const ptrdiff_t *no,
                                 ptrdiff_t howmany, const ptrdiff_t *iblock, const ptrdiff_t *oblock, double *in,
                                 pfft_complex *out, MPI_Comm comm_cart, int sign, unsigned pfft_flags) {
  (void)rnk; (void)n; (void)ni; (void)no; (void)howmany; (void)iblock; (void)oblock; (void)in; (void)out;
  (void)comm_cart; (void)sign; (void)pfft_flags;
  die("the r2c transforms");
  return NULL;
}

/* out[l] = sum_k in[k] exp(sign 2 pi i k.l / n): the ni-block (k_t from
 * -ni_t/2) zero-padded onto the n-grid at k mod n, transformed, and the
 * no-block (l_t from -no_t/2) read at l mod n */
void pfft_execute(const pfft_plan p) {
  const ptrdiff_t n0 = p->n[0], n1 = p->n[1], n2 = p->n[2];
  pfft_complex *g = (pfft_complex *)calloc((size_t)(n0 * n1 * n2), sizeof(pfft_complex));
  ptrdiff_t mx = n0 > n1 ? n0 : n1;
  mx = mx > n2 ? mx : n2;
  pfft_complex *tmp = (pfft_complex *)malloc(sizeof(pfft_complex) * (size_t)mx);
  for (ptrdiff_t a = 0; a < p->ni[0]; a++)
    for (ptrdiff_t b = 0; b < p->ni[1]; b++)
      for (ptrdiff_t c = 0; c < p->ni[2]; c++) {
        const ptrdiff_t k0 = wrapn(a - p->ni[0] / 2, n0), k1 = wrapn(b - p->ni[1] / 2, n1),
                        k2 = wrapn(c - p->ni[2] / 2, n2);
        g[(k0 * n1 + k1) * n2 + k2] += p->in[(a * p->ni[1] + b) * p->ni[2] + c];
      }
  for (ptrdiff_t a = 0; a < n0; a++)
    for (ptrdiff_t b = 0; b < n1; b++) dft1(g + (a * n1 + b) * n2, n2, 1, p->sign, tmp);
  for (ptrdiff_t a = 0; a < n0; a++)
    for (ptrdiff_t c = 0; c < n2; c++) dft1(g + a * n1 * n2 + c, n1, n2, p->sign, tmp);
  for (ptrdiff_t b = 0; b < n1; b++)
    for (ptrdiff_t c = 0; c < n2; c++) dft1(g + b * n2 + c, n0, n1 * n2, p->sign, tmp);
  for (ptrdiff_t a = 0; a < p->no[0]; a++)
    for (ptrdiff_t b = 0; b < p->no[1]; b++)
      for (ptrdiff_t c = 0; c < p->no[2]; c++) {
        const ptrdiff_t l0 = wrapn(a - p->no[0] / 2, n0), l1 = wrapn(b - p->no[1] / 2, n1),
                        l2 = wrapn(c - p->no[2] / 2, n2);
        p->out[(a * p->no[1] + b) * p->no[2] + c] = g[(l0 * n1 + l1) * n2 + l2];
      }
  free(tmp);
  free(g);
}
void pfft_destroy_plan(pfft_plan p) { free(p); }

/* ------------------------------------------------------------------------- */
/* PFFT: periodic ghost cells on one process                                 */
/* ------------------------------------------------------------------------- */
struct pfft_gcplan_s {
  ptrdiff_t n[3], below[3], above[3];
  pfft_complex *data;
};

ptrdiff_t pfft_local_size_many_gc(int rnk, const ptrdiff_t *local_n, const ptrdiff_t *local_start,
                                  ptrdiff_t howmany, const ptrdiff_t *gc_below, const ptrdiff_t *gc_above,
                                  ptrdiff_t *local_ngc, ptrdiff_t *local_gc_start) {
  for (int t = 0; t < rnk; t++) {
    local_ngc[t] = local_n[t] + gc_below[t] + gc_above[t];
    local_gc_start[t] = local_start[t] - gc_below[t];
  }
  return howmany * pfft_prod_INT(rnk, local_ngc);
}
pfft_gcplan pfft_plan_many_cgc(int rnk, const ptrdiff_t *n, ptrdiff_t howmany, const ptrdiff_t *block,
                               const ptrdiff_t *gc_below, const ptrdiff_t *gc_above, pfft_complex *data,
                               MPI_Comm comm_cart, unsigned gc_flags) {
  (void)block; (void)comm_cart; (void)gc_flags;
  if (rnk != 3 || howmany != 1) die("this ghost-cell rank or howmany");
  struct pfft_gcplan_s *p = (struct pfft_gcplan_s *)calloc(1, sizeof(*p));
  for (int t = 0; t < 3; t++) {
    p->n[t] = n[t];
    p->below[t] = gc_below[t];
    p->above[t] = gc_above[t];
  }
  p->data = data;
  return p;
}
pfft_gcplan pfft_plan_many_rgc(int rnk, const ptrdiff_t *n, ptrdiff_t howmany, const ptrdiff_t *block,
                               const ptrdiff_t *gc_below, const ptrdiff_t *gc_above, double *data,
                               MPI_Comm comm_cart, unsigned gc_flags) {
  (void)rnk; (void)n; (void)howmany; (void)block; (void)gc_below; (void)gc_above; (void)data; (void)comm_cart;
  (void)gc_flags;
  die("the real ghost cells");
  return NULL;
}

/* ghost-celled block a_t in [0, n_t + below_t + above_t) holds the value of
 * the block point (a_t - below_t) mod n_t */
void pfft_exchange(pfft_gcplan p) {
  const ptrdiff_t n0 = p->n[0], n1 = p->n[1], n2 = p->n[2];
  const ptrdiff_t g0 = n0 + p->below[0] + p->above[0], g1 = n1 + p->below[1] + p->above[1],
                  g2 = n2 + p->below[2] + p->above[2];
  const size_t nb = (size_t)(n0 * n1 * n2);
  pfft_complex *old = (pfft_complex *)malloc(sizeof(pfft_complex) * nb);
  memcpy(old, p->data, sizeof(pfft_complex) * nb);
  for (ptrdiff_t a = 0; a < g0; a++)
    for (ptrdiff_t b = 0; b < g1; b++)
      for (ptrdiff_t c = 0; c < g2; c++) {
        const ptrdiff_t o0 = wrapn(a - p->below[0], n0), o1 = wrapn(b - p->below[1], n1),
                        o2 = wrapn(c - p->below[2], n2);
        p->data[(a * g1 + b) * g2 + c] = old[(o0 * n1 + o1) * n2 + o2];
      }
  free(old);
}
/* the transpose: every ghost-celled point is added onto its block point */
void pfft_reduce(pfft_gcplan p) {
  const ptrdiff_t n0 = p->n[0], n1 = p->n[1], n2 = p->n[2];
  const ptrdiff_t g0 = n0 + p->below[0] + p->above[0], g1 = n1 + p->below[1] + p->above[1],
                  g2 = n2 + p->below[2] + p->above[2];
  const size_t nb = (size_t)(n0 * n1 * n2);
  pfft_complex *acc = (pfft_complex *)calloc(nb, sizeof(pfft_complex));
  for (ptrdiff_t a = 0; a < g0; a++)
    for (ptrdiff_t b = 0; b < g1; b++)
      for (ptrdiff_t c = 0; c < g2; c++) {
        const ptrdiff_t o0 = wrapn(a - p->below[0], n0), o1 = wrapn(b - p->below[1], n1),
                        o2 = wrapn(c - p->below[2], n2);
        acc[(o0 * n1 + o1) * n2 + o2] += p->data[(a * g1 + b) * g2 + c];
      }
  memcpy(p->data, acc, sizeof(pfft_complex) * nb);
  free(acc);
}
void pfft_destroy_gcplan(pfft_gcplan p) { free(p); }
