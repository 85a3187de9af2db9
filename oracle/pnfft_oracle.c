/*
 * pnfft_oracle.c -- CPU restatement (FP64) of the PNFFT hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker against which the CUDA
 * library is compared; it is loaded by tests/, by __graft_entry__.smoke() and
 * by the CPU legs of bench.py.  Nothing in the product (pnfft_gb300/, include/)
 * links it or calls it.
 *
 * Every routine restates the arithmetic of the reference (mpip/pnfft 1.0.7-alpha)
 * for a single-process 1x1x1 mesh and names the reference lines it follows.
 * Differences in *storage* (not arithmetic):
 *   - the oversampled grid is kept in natural FFT order (index l mod n) instead
 *     of PFFT's shifted array with m ghost planes; for nodes in [-0.5,0.5)^3 the
 *     periodic ghost-cell copy/add of the reference (kernel/ndft-parallel.c:2558,
 *     2679) is the same as this modulo wrap;
 *   - the F step itself (PFFT zero-pad + FFT, ndft-parallel.c:1524-1546) is done
 *     by the Python driver oracle/pnfft_oracle.py with scipy.fft.
 * Third-party arithmetic the reference takes from libraries outside its tree
 * is restated from its published definition:
 *   GSL gsl_sf_bessel_I0/I1 (kernel/bessel_i0.c:375, bessel_i1.c:570) -> power
 *   series; libcerf cerf() for PNFFT_WINDOW_GAUSSIAN_T (kernel/matrix_D.c:43)
 *   -> Re erf(a+iy) by quadrature of its defining integral.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;
typedef int64_t I64;

/* plan flags (api/pnfft.h:302-334) */
#define F_PRE_PHI_HAT (1u << 0)
#define F_FAST_GAUSSIAN (1u << 1)
#define F_PRE_CONST_PSI (1u << 2)
#define F_PRE_LIN_PSI (1u << 3)
#define F_PRE_QUAD_PSI (1u << 4)
#define F_PRE_CUB_PSI (1u << 5)
#define F_PRE_INTPOL (F_PRE_CONST_PSI | F_PRE_LIN_PSI | F_PRE_QUAD_PSI | F_PRE_CUB_PSI)
#define F_INTERLACED (1u << 8)
#define F_TRANSPOSED (1u << 11)
#define F_DIFF_IK (1u << 12)
#define F_WIN_GAUSS (1u << 13)
#define F_WIN_BSPLINE (1u << 14)
#define F_WIN_SINC (1u << 15)
#define F_WIN_I0 (1u << 16)
#define F_GAUSS_T (1u << 17)
#define F_REAL_F (1u << 4) /* node flag tested against plan flags, ndft-parallel.c:2804 */
/* compute flags (api/pnfft.h:383-390) */
#define C_F (1u << 0)
#define C_GRAD (1u << 1)
#define C_HESS (1u << 2)

static const double PI = 3.14159265358979323846;

typedef struct or_plan_s {
  I64 N[3], n[3];
  int m, cutoff, c2r;
  unsigned flags;
  double b[3], sigma[3];
  int intpol_order;
  I64 intpol_K;
  double *tab[3][3]; /* [derivative][dim] */
  double exp_const[3][64];
} or_plan;

/* ---------------------------------------------------------------------------
 * special functions
 * ------------------------------------------------------------------------- */

/* modified Bessel I0 by its power series sum_k (x^2/4)^k / (k!)^2 (all terms
 * positive, so the sum is accurate to a few ulp); stands in for GSL's I0. */
double or_bessel_i0(double x) {
  double q = 0.25 * x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k < 500; k++) {
    term *= q / ((double)k * (double)k);
    sum += term;
    if (term < 1e-18 * sum) break;
  }
  return sum;
}

/* modified Bessel I1: sum_k (x/2)^(2k+1) / (k! (k+1)!) */
double or_bessel_i1(double x) {
  double q = 0.25 * x * x, term = 0.5 * x, sum = term;
  for (int k = 1; k < 500; k++) {
    term *= q / ((double)k * (double)(k + 1));
    sum += term;
    if (fabs(term) < 1e-18 * fabs(sum)) break;
  }
  return sum;
}

/* Re erf(a + i y) = erf(a) + 2/sqrt(pi) e^{-a^2} int_0^y e^{t^2} sin(2 a t) dt,
 * the integral by composite 16-point Gauss-Legendre (nodes computed by Newton). */
static double gl_x[16], gl_w[16];
static int gl_ready = 0;
static void gl_init(void) {
  const int n = 16;
  for (int i = 0; i < n; i++) {
    double z = cos(PI * (i + 0.75) / (n + 0.5)), pp = 0;
    for (int it = 0; it < 100; it++) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; j++) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      double z1 = z;
      z = z1 - p1 / pp;
      if (fabs(z - z1) < 1e-16) break;
    }
    gl_x[i] = z;
    gl_w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
  gl_ready = 1;
}
double or_re_erf_complex(double a, double y) {
  if (!gl_ready) gl_init();
  int panels = 32;
  double h = y / panels, s = 0;
  for (int p = 0; p < panels; p++) {
    double c = (p + 0.5) * h;
    for (int i = 0; i < 16; i++) {
      double t = c + 0.5 * h * gl_x[i];
      s += gl_w[i] * 0.5 * h * exp(t * t - a * a) * sin(2.0 * a * t);
    }
  }
  return erf(a) + 2.0 / sqrt(PI) * s;
}

/* sinc with small-argument branches, kernel/sinc.c:26-53 */
static double or_sinc(double x) {
  const double e = 2.220446049250313e-16, es = sqrt(e), es2 = sqrt(es);
  if (fabs(x) >= es2) return sin(x) / x;
  double r = 1.0;
  if (fabs(x) >= e) {
    double x2 = x * x;
    r -= x2 / 6.0;
    if (fabs(x) >= es) r += x2 * x2 / 120.0;
  }
  return r;
}

/* Cardinal B-spline of order p, M_p supported on (0,p): the values
 * M_p(phi + i), i = 0..p-1, for phi in [0,1], by the Cox-de Boor recursion
 * M_k(t) = (t M_{k-1}(t) + (k-t) M_{k-1}(t-1)) / (k-1).  (The reference uses
 * de Boor's scheme, kernel/bspline.c:45-91, and per-order polynomial pieces,
 * bspline.c:94-670; both evaluate this same function.) */
static void bspline_pieces(int p, double phi, double *out) {
  double v[64];
  v[0] = 1.0;
  for (int k = 2; k <= p; k++) {
    double nv[64];
    for (int i = 0; i < k; i++) {
      double t = phi + i;
      double a = (i <= k - 2) ? v[i] : 0.0;
      double b = (i >= 1) ? v[i - 1] : 0.0;
      nv[i] = (t * a + (k - t) * b) / (k - 1);
    }
    memcpy(v, nv, sizeof(double) * k);
  }
  memcpy(out, v, sizeof(double) * p);
}

/* M_p(x), zero outside the open interval (0,p) -- PNX(bspline), bspline.c:45 */
double or_bspline(int p, double x) {
  if (p < 1 || !(0 < x && x < p)) return 0.0;
  if (p - x < x) x = p - x;
  double fl = floor(x), phi = x - fl;
  int j = (int)fl;
  double v[64];
  bspline_pieces(p, phi, v);
  return v[j];
}

/* ---------------------------------------------------------------------------
 * 1-D windows psi(x) and derivatives, kernel/ndft-parallel.c:2194-2464
 * ------------------------------------------------------------------------- */
static double kb_psi(double x, I64 n, double b, int m) { /* 2241-2254 */
  double d = (double)m * m - (x * n) * (x * n);
  double r = (d < 0) ? sqrt(-d) : sqrt(d);
  if (d < 0) return sin(b * r) / (PI * r);
  return (d > 0) ? sinh(b * r) / (PI * r) : b / PI;
}
static double kb_dpsi(double x, I64 n, double b, int m, double psi) { /* 2256-2269 */
  double d = (double)m * m - (x * n) * (x * n);
  double r = (d < 0) ? sqrt(-d) : sqrt(d);
  if (d < 0) return n * n * x / d * (psi - b * cos(b * r) / PI);
  return (d > 0) ? n * n * x / d * (psi - b * cosh(b * r) / PI) : -n * m * b * b * b / (3.0 * PI);
}
static double kb_ddpsi(double x, I64 n, double b, int m, double psi, double dpsi) { /* 2272-2285 */
  double d = (double)m * m - (x * n) * (x * n);
  double r = (d < 0) ? sqrt(-d) : sqrt(d);
  double bnx = b * n * x;
  if (d < 0)
    return 3.0 * n * n * x * dpsi / d + n * n * psi / d * (1.0 + bnx * bnx) - b * n * n / (PI * d) * cos(b * r);
  if (d > 0)
    return 3.0 * n * n * x * dpsi / d + n * n * psi / d * (1.0 + bnx * bnx) - b * n * n / (PI * d) * cosh(b * r);
  double bn = b * n, bm = b * m;
  return b * bn * bn / (15.0 * PI) * (bm * bm - 5.0);
}
static double i0w_psi(double x, I64 n, double b, int m) { /* 2195-2203 */
  double d = (double)m * m - (x * n) * (x * n);
  return (d < 0) ? 0.0 : 0.5 * or_bessel_i0(b * sqrt(d));
}
static double i0w_dpsi(double x, I64 n, double b, int m) { /* 2205-2218 */
  double d = (double)m * m - (x * n) * (x * n);
  double r = (d < 0) ? sqrt(-d) : sqrt(d);
  if (d < 0) return 0.0;
  if (d > 0) return -0.5 * b * (double)n * (double)n * x * or_bessel_i1(b * r) / r;
  double h = 0.5 * b * n;
  return -h * h * x;
}
static double i0w_ddpsi(double x, I64 n, double b, int m) { /* 2220-2239 */
  double d = (double)m * m - (x * n) * (x * n);
  double r = (d < 0) ? sqrt(-d) : sqrt(d);
  if (d < 0) return 0.0;
  if (d > 0) {
    double y = ((double)n * x) * ((double)n * x);
    return 0.5 * b * (double)n * (double)n / d * (b * y * or_bessel_i0(b * r) - or_bessel_i1(b * r) / r * (y + m * m));
  }
  double t1 = b * b * (double)m * (double)n, t2 = b * (double)n;
  return t1 * t1 / 16.0 - t2 * t2 / 4.0;
}
static double gauss_psi(double x, I64 n, double b) { /* 2337-2342 */
  return exp(-(n * x) * (n * x) / b) / sqrt(PI * b);
}
static double gauss_dpsi(double x, I64 n, double b) { /* 2344-2349 */
  return -2.0 * n / b * n * x * exp(-(n * x) * (n * x) / b) / sqrt(PI * b);
}
static double gauss_ddpsi(double x, I64 n, double b) { /* 2351-2357 */
  double y = (n * x) * (n * x) / b;
  return 2.0 * n / b * n * exp(-y) / sqrt(PI * b) * (2.0 * y - 1.0);
}
static double sincp_psi(double x, I64 n, double b, int m) { /* 2386-2395 */
  return pow(or_sinc(PI * (n * x) / b), 2.0 * m) / b;
}
static double sincp_dpsi(double x, I64 n, double b, int m) { /* 2397-2406 */
  double y = PI * n * x / b;
  if (fabs(y) > 2.220446049250313e-16)
    return 2.0 * m * PI * (double)n / b * (1.0 / tan(y) - 1.0 / y) * sincp_psi(x, n, b, m);
  return 0.0;
}
static double sincp_ddpsi(double x, I64 n, double b, int m) { /* 2408-2418 */
  double y = PI * n * x / b, q = PI * (double)n / b;
  if (fabs(y) > 2.220446049250313e-16) {
    double ty = tan(y);
    return 2.0 * m * PI * (double)n / b * (1.0 / ty - 1.0 / y) * sincp_dpsi(x, n, b, m) +
           2.0 * m * q * q * (-1.0 + 1.0 / (y * y) - 1.0 / (ty * ty)) * sincp_psi(x, n, b, m);
  }
  return -2.0 * m / (3.0 * b) * q * q;
}
static double bspl_psi(double x, I64 n, int m) { return or_bspline(2 * m, n * x + m); } /* 2359-2365 */
static double bspl_dpsi(double x, I64 n, int m) {                                      /* 2367-2374 */
  return (double)n * (or_bspline(2 * m - 1, n * x + m) - or_bspline(2 * m - 1, n * x + m - 1));
}
static double bspl_ddpsi(double x, I64 n, int m) { /* 2376-2384 */
  return (double)n * (double)n *
         (or_bspline(2 * m - 2, n * x + m) - 2.0 * or_bspline(2 * m - 2, n * x + m - 1) + or_bspline(2 * m - 2, n * x + m - 2));
}

/* PNX(psi/dpsi/ddpsi) dispatch, ndft-parallel.c:2288-2334 */
double or_psi(const or_plan *p, int t, double x) {
  unsigned f = p->flags;
  if (f & F_WIN_GAUSS) return gauss_psi(x, p->n[t], p->b[t]);
  if (f & F_WIN_BSPLINE) return bspl_psi(x, p->n[t], p->m);
  if (f & F_WIN_SINC) return sincp_psi(x, p->n[t], p->b[t], p->m);
  if (f & F_WIN_I0) return i0w_psi(x, p->n[t], p->b[t], p->m);
  return kb_psi(x, p->n[t], p->b[t], p->m);
}
double or_dpsi(const or_plan *p, int t, double x) {
  unsigned f = p->flags;
  if (f & F_WIN_GAUSS) return gauss_dpsi(x, p->n[t], p->b[t]);
  if (f & F_WIN_BSPLINE) return bspl_dpsi(x, p->n[t], p->m);
  if (f & F_WIN_SINC) return sincp_dpsi(x, p->n[t], p->b[t], p->m);
  if (f & F_WIN_I0) return i0w_dpsi(x, p->n[t], p->b[t], p->m);
  return kb_dpsi(x, p->n[t], p->b[t], p->m, kb_psi(x, p->n[t], p->b[t], p->m));
}
double or_ddpsi(const or_plan *p, int t, double x) {
  unsigned f = p->flags;
  if (f & F_WIN_GAUSS) return gauss_ddpsi(x, p->n[t], p->b[t]);
  if (f & F_WIN_BSPLINE) return bspl_ddpsi(x, p->n[t], p->m);
  if (f & F_WIN_SINC) return sincp_ddpsi(x, p->n[t], p->b[t], p->m);
  if (f & F_WIN_I0) return i0w_ddpsi(x, p->n[t], p->b[t], p->m);
  double ps = kb_psi(x, p->n[t], p->b[t], p->m);
  double dps = kb_dpsi(x, p->n[t], p->b[t], p->m, ps);
  return kb_ddpsi(x, p->n[t], p->b[t], p->m, ps, dps);
}

/* ---------------------------------------------------------------------------
 * window Fourier coefficients, kernel/matrix_D.c:30-225
 * ------------------------------------------------------------------------- */
double or_phi_hat(const or_plan *p, int t, I64 k) {
  unsigned f = p->flags;
  I64 n = p->n[t];
  double b = p->b[t];
  int m = p->m;
  if ((f & F_WIN_GAUSS) && (f & F_GAUSS_T)) { /* 57-64 */
    double sb = sqrt(b), q = PI * (double)k / (double)n;
    return exp(-q * q * b) * or_re_erf_complex((double)m / sb, PI * (double)k * sb / (double)n);
  }
  if (f & F_WIN_GAUSS) { /* 33-34 */
    double q = PI * (double)k / (double)n;
    return exp(-q * q * b);
  }
  if (f & F_WIN_BSPLINE) return pow(or_sinc((double)k * PI / (double)n), 2.0 * m); /* 121-122 */
  if (f & F_WIN_SINC) return or_bspline(2 * m, fabs((double)k * b / (double)n) + m); /* 134-140 */
  double q = 2.0 * PI * (double)k / (double)n;
  double d = b * b - q * q;
  if (f & F_WIN_I0) { /* 104-115 */
    double r = (d < 0) ? sqrt(-d) : sqrt(d);
    if (d < 0) return sin(m * r) / r;
    return (d > 0) ? sinh(m * r) / r : (double)m;
  }
  if (d < 0) return 0.0; /* 79-89 */
  return (d > 0) ? or_bessel_i0(m * sqrt(d)) : 1.0;
}

double or_inv_phi_hat(const or_plan *p, int t, I64 k) {
  unsigned f = p->flags;
  I64 n = p->n[t];
  double b = p->b[t];
  int m = p->m;
  if ((f & F_WIN_GAUSS) && (f & F_GAUSS_T)) return 1.0 / or_phi_hat(p, t, k); /* 37-55 */
  if (f & F_WIN_GAUSS) {                                                       /* 30-31 */
    double q = PI * (double)k / (double)n;
    return exp(q * q * b);
  }
  if (f & F_WIN_BSPLINE) return pow(or_sinc((double)k * PI / (double)n), -2.0 * m); /* 118-119 */
  if (f & F_WIN_SINC) {                                                              /* 124-132 */
    double d = fabs((double)k * b / (double)n);
    return (d < m) ? 1.0 / or_bspline(2 * m, d + m) : 0.0;
  }
  double q = 2.0 * PI * (double)k / (double)n;
  double d = b * b - q * q;
  if (f & F_WIN_I0) { /* 91-102 */
    double r = (d < 0) ? sqrt(-d) : sqrt(d);
    if (d < 0) return r / sin(m * r);
    return (d > 0) ? r / sinh(m * r) : 1.0 / m;
  }
  if (d < 0) return 0.0; /* 66-77 */
  return (d > 0) ? 1.0 / or_bessel_i0(m * sqrt(d)) : 1.0;
}

/* ---------------------------------------------------------------------------
 * plan set-up: window shape b (ndft-parallel.c:1008-1064), fast-Gaussian
 * constants and interpolation tables (1072-1122, 321-353)
 * ------------------------------------------------------------------------- */
static void build_tables(or_plan *p) {
  for (int d = 0; d < 3; d++)
    for (int t = 0; t < 3; t++) {
      free(p->tab[d][t]);
      p->tab[d][t] = NULL;
    }
  if (p->flags & F_FAST_GAUSSIAN)
    for (int t = 0; t < 3; t++)
      for (int s = 0; s < p->cutoff && s < 64; s++)
        p->exp_const[t][s] = exp(-(double)(s * s) / p->b[t]) / sqrt(PI * p->b[t]);
  if (!(p->flags & F_PRE_INTPOL)) return;
  int ord = p->intpol_order;
  I64 K = (I64)ceil((2.0 * 15.0 + 1.0) / p->cutoff) * 2048; /* 1095 */
  p->intpol_K = K;
  int nder = (p->flags & F_DIFF_IK) ? 1 : 3; /* 1105 */
  for (int der = 0; der < nder; der++)
    for (int t = 0; t < 3; t++) {
      I64 sz = K * p->cutoff * (ord + 1);
      double *tab = (double *)malloc(sizeof(double) * sz);
      I64 ind = 0;
      for (I64 k = 0; k < K; k++)
        for (int c = 0; c < p->cutoff; c++)
          for (int i = -ord / 2; i <= (ord + 1) / 2; i++, ind++) {
            double arg = (p->m + (double)(k + i) / K - c) / p->n[t];
            if (der == 0) tab[ind] = or_psi(p, t, arg);
            else if (der == 1) tab[ind] = or_dpsi(p, t, arg);
            else tab[ind] = or_ddpsi(p, t, arg);
          }
      p->tab[der][t] = tab;
    }
}

or_plan *or_plan_create(const I64 *N, const I64 *n, int m, unsigned flags, int c2r) {
  or_plan *p = (or_plan *)calloc(1, sizeof(or_plan));
  for (int t = 0; t < 3; t++) {
    p->N[t] = N[t];
    p->n[t] = n[t];
    p->sigma[t] = (double)n[t] / (double)N[t];
  }
  /* flag promotion of api/api-guru.c:152-155: the precompute-flag values
   * PRE_HESSIAN_PSI (1<<3) and PRE_GRAD_PSI (1<<2) are tested on plan flags */
  if (flags & (1u << 3)) flags |= (1u << 2);
  if (flags & (1u << 2)) flags |= (1u << 1);
  p->flags = flags;
  p->m = m;
  p->cutoff = 2 * m + 1;
  p->c2r = c2r;
  if (flags & F_PRE_CONST_PSI) p->intpol_order = 0; /* 997-1006 */
  else if (flags & F_PRE_LIN_PSI) p->intpol_order = 1;
  else if (flags & F_PRE_QUAD_PSI) p->intpol_order = 2;
  else if (flags & F_PRE_CUB_PSI) p->intpol_order = 3;
  else p->intpol_order = -1;
  for (int t = 0; t < 3; t++) {
    double s = p->sigma[t];
    if (flags & F_WIN_GAUSS) p->b[t] = ((double)m / PI) * 2.0 * s / (2.0 * s - 1.0); /* 1015 */
    else if (flags & F_WIN_BSPLINE) p->b[t] = 0.0;
    else if (flags & F_WIN_SINC) p->b[t] = (double)m * (2.0 * s) / (2.0 * s - 1.0); /* 1043 */
    else p->b[t] = PI * (2.0 - 1.0 / s);                                             /* 1052, 1059 */
  }
  build_tables(p);
  return p;
}

void or_plan_destroy(or_plan *p) {
  if (!p) return;
  for (int d = 0; d < 3; d++)
    for (int t = 0; t < 3; t++) free(p->tab[d][t]);
  free(p);
}

void or_set_b(or_plan *p, double b0, double b1, double b2) { /* api-basic.c:587-596 */
  p->b[0] = b0;
  p->b[1] = b1;
  p->b[2] = b2;
  build_tables(p);
}
double or_get_b(const or_plan *p, int t) { return p->b[t]; }
unsigned or_get_flags(const or_plan *p) { return p->flags; }
I64 or_intpol_K(const or_plan *p) { return p->intpol_K; }
int or_intpol_order(const or_plan *p) { return p->intpol_order; }
const double *or_table(const or_plan *p, int der, int t) { return p->tab[der][t]; }

/* ---------------------------------------------------------------------------
 * window values on the 3 axes of one node, ndft-parallel.c:1586-2105
 *   x: node (already shifted for interlacing), fnx: floor(n x) per axis
 *   out[cutoff*t + s] for the grid point floor(n_t x_t) - m + s
 * ------------------------------------------------------------------------- */
static void tensor_intpol(const or_plan *p, const double *x, const double *fnx, double *const *tabs, double *out) {
  /* 1586-1617 and ipnfft.h:457-500 */
  int cut = p->cutoff, ord = p->intpol_order;
  I64 K = p->intpol_K;
  for (int t = 0; t < 3; t++) {
    double dist = p->n[t] * x[t] - fnx[t];
    I64 k = (I64)floor(dist * K);
    double dk = dist * K - (double)k;
    k *= cut * (ord + 1);
    const double *T = tabs[t];
    for (int s = 0; s < cut; s++, k += ord + 1) {
      double v;
      if (ord == 0) v = T[k];
      else if (ord == 1) v = T[k] * (1.0 - dk) + T[k + 1] * dk;
      else if (ord == 2) {
        double f0 = T[k], f1 = T[k + 1], f2 = T[k + 2], c0 = dk + 1.0, c1 = dk, c2 = dk - 1.0;
        v = 0.5 * f0 * c1 * c2 - c0 * f1 * c2 + 0.5 * c0 * c1 * f2;
      } else {
        double f0 = T[k], f1 = T[k + 1], f2 = T[k + 2], f3 = T[k + 3];
        double c0 = dk + 1.0, c1 = dk, c2 = dk - 1.0, c3 = dk - 2.0;
        v = (-f0 * c1 * c2 * c3 + 3.0 * c0 * f1 * c2 * c3 - 3.0 * c0 * c1 * f2 * c3 + c0 * c1 * c2 * f3) / 6.0;
      }
      out[cut * t + s] = v;
    }
  }
}

static void tensor_psi(const or_plan *p, const double *x, const double *fnx, double *psi) {
  int cut = p->cutoff, m = p->m;
  unsigned f = p->flags;
  if (f & F_PRE_INTPOL) {
    double *const tabs[3] = {p->tab[0][0], p->tab[0][1], p->tab[0][2]};
    tensor_intpol(p, x, fnx, tabs, psi);
    return;
  }
  for (int t = 0; t < 3; t++) {
    I64 n = p->n[t];
    double b = p->b[t];
    double *o = psi + cut * t;
    if (f & F_WIN_GAUSS) {
      if (f & F_FAST_GAUSSIAN) { /* 1694-1714 */
        double uj = fnx[t] - m;
        double a = n * x[t] - uj;
        double es = exp(-a * a / b), el = exp(2.0 * a / b), tmp = es;
        for (int s = 0; s < cut; s++) {
          o[s] = tmp * p->exp_const[t][s];
          tmp *= el;
        }
      } else { /* 1678-1692 */
        double uj = fnx[t] - n * x[t] - m;
        for (int s = 0; s < cut; s++) o[s] = exp(-(uj + s) * (uj + s) / b) / sqrt(PI * b);
      }
    } else if (f & F_WIN_BSPLINE) { /* 1716-1742: M_{2m}(fnx - n x + s) */
      double phi = 1.0 - (n * x[t] - fnx[t]);
      double v[64];
      bspline_pieces(2 * m, phi, v);
      o[0] = 0.0;
      for (int s = 1; s < cut; s++) o[s] = v[s - 1];
    } else if (f & F_WIN_SINC) { /* 1745-1763 */
      double uj = fnx[t] - n * x[t] - m;
      for (int s = 0; s < cut; s++) o[s] = pow(or_sinc(PI * (uj + s) / b), 2.0 * m) / b;
    } else if (f & F_WIN_I0) { /* 1765-1780 */
      double uj = fnx[t] - n * x[t] - m;
      for (int s = 0; s < cut; s++) o[s] = i0w_psi((uj + s) / n, n, b, m);
    } else { /* 1782-1797 */
      double uj = fnx[t] - n * x[t] - m;
      for (int s = 0; s < cut; s++) o[s] = kb_psi((uj + s) / n, n, b, m);
    }
  }
}

static void tensor_dpsi(const or_plan *p, const double *x, const double *fnx, const double *psi, double *dpsi) {
  int cut = p->cutoff, m = p->m;
  unsigned f = p->flags;
  if (f & F_PRE_INTPOL) {
    double *const tabs[3] = {p->tab[1][0], p->tab[1][1], p->tab[1][2]};
    tensor_intpol(p, x, fnx, tabs, dpsi);
    return;
  }
  for (int t = 0; t < 3; t++) {
    I64 n = p->n[t];
    double b = p->b[t];
    double *o = dpsi + cut * t;
    const double *ps = psi + cut * t;
    double uj = n * x[t] - fnx[t] + m;
    if (f & F_WIN_GAUSS) { /* 1850-1864 */
      for (int s = 0; s < cut; s++) o[s] = -2.0 * n / b * (uj - s) * ps[s];
    } else if (f & F_WIN_BSPLINE) { /* 1866-1893: d/dx M_{2m}(fnx - n x + s) */
      double phi = 1.0 - (n * x[t] - fnx[t]);
      double v[64];
      bspline_pieces(2 * m - 1, phi, v);
      for (int s = 0; s < cut; s++) {
        /* M'_{2m}(t) = M_{2m-1}(t) - M_{2m-1}(t-1), t = phi + s - 1 */
        double a = (s - 1 >= 0 && s - 1 < 2 * m - 1) ? v[s - 1] : 0.0;
        double c = (s - 2 >= 0 && s - 2 < 2 * m - 1) ? v[s - 2] : 0.0;
        o[s] = -(double)n * (a - c);
      }
    } else if (f & F_WIN_SINC) { /* 1897-1917 */
      for (int s = 0; s < cut; s++) {
        double y = PI * (uj - s) / b;
        o[s] = (fabs(y) > 2.220446049250313e-16) ? 2.0 * m * PI * (double)n / b * (1.0 / tan(y) - 1.0 / y) * ps[s] : 0.0;
      }
    } else if (f & F_WIN_I0) { /* 1919-1934 */
      for (int s = 0; s < cut; s++) o[s] = i0w_dpsi((uj - s) / n, n, b, m);
    } else { /* 1937-1953 */
      for (int s = 0; s < cut; s++) o[s] = kb_dpsi((uj - s) / n, n, b, m, ps[s]);
    }
  }
}

static void tensor_ddpsi(const or_plan *p, const double *x, const double *fnx, const double *psi, const double *dpsi, double *ddpsi) {
  int cut = p->cutoff, m = p->m;
  unsigned f = p->flags;
  if (f & F_PRE_INTPOL) {
    double *const tabs[3] = {p->tab[2][0], p->tab[2][1], p->tab[2][2]};
    tensor_intpol(p, x, fnx, tabs, ddpsi);
    return;
  }
  for (int t = 0; t < 3; t++) {
    I64 n = p->n[t];
    double b = p->b[t];
    double *o = ddpsi + cut * t;
    const double *ps = psi + cut * t, *dps = dpsi + cut * t;
    double uj = n * x[t] - fnx[t] + m;
    if (f & F_WIN_GAUSS) { /* 2006-2020 */
      for (int s = 0; s < cut; s++) o[s] = 2.0 * n * n / b * (2.0 / b * (uj - s) * (uj - s) - 1.0) * ps[s];
    } else if (f & F_WIN_BSPLINE) { /* 2022-2049 */
      double phi = 1.0 - (n * x[t] - fnx[t]);
      double v[64];
      int q = 2 * m - 2;
      if (q >= 1) bspline_pieces(q, phi, v);
      for (int s = 0; s < cut; s++) {
        double a = (q >= 1 && s - 1 >= 0 && s - 1 < q) ? v[s - 1] : 0.0;
        double c = (q >= 1 && s - 2 >= 0 && s - 2 < q) ? v[s - 2] : 0.0;
        double e = (q >= 1 && s - 3 >= 0 && s - 3 < q) ? v[s - 3] : 0.0;
        o[s] = (double)n * (double)n * (a - 2.0 * c + e);
      }
    } else if (f & F_WIN_SINC) { /* 2052-2072 */
      double qq = PI * (double)n / b;
      for (int s = 0; s < cut; s++) {
        double y = PI * (uj - s) / b;
        if (fabs(y) > 2.220446049250313e-16) {
          double ty = tan(y);
          o[s] = 2.0 * m * PI * (double)n / b * (1.0 / ty - 1.0 / y) * dps[s] +
                 2.0 * m * qq * qq * (1.0 / (y * y) - 1.0 - 1.0 / (ty * ty)) * ps[s];
        } else
          o[s] = -2.0 * m * qq * qq / (3.0 * b);
      }
    } else if (f & F_WIN_I0) { /* 2074-2089 */
      for (int s = 0; s < cut; s++) o[s] = i0w_ddpsi((uj - s) / n, n, b, m);
    } else { /* 2091-2105 */
      for (int s = 0; s < cut; s++) o[s] = kb_ddpsi((uj - s) / n, n, b, m, ps[s], dps[s]);
    }
  }
}

/* node position after the optional interlacing shift, the grid index
 * floor(n x) - m and the fold back into [-0.5,0.5), ndft-parallel.c:2732-2753 */
static void node_setup(const or_plan *p, const double *xj, int interlaced, double *x, double *fnx, I64 *u) {
  for (int t = 0; t < 3; t++) {
    x[t] = xj[t];
    if (interlaced) x[t] += 0.5 / p->n[t];
  }
  for (int t = 0; t < 3; t++) { /* 1563-1572, 2165-2174 */
    fnx[t] = floor(p->n[t] * x[t]);
    u[t] = (I64)fnx[t] - p->m;
  }
  if (interlaced)
    for (int t = 0; t < 3; t++)
      if (x[t] >= 0.5) {
        x[t] -= 1.0;
        fnx[t] -= p->n[t];
      }
}

/* exported for bit-exact index tests: floor(n x) and fold, per node */
void or_node_index(const or_plan *p, I64 M, const double *x, int interlaced, I64 *u_out, double *fnx_out) {
  for (I64 j = 0; j < M; j++) {
    double xs[3], fnx[3];
    I64 u[3];
    node_setup(p, x + 3 * j, interlaced, xs, fnx, u);
    for (int t = 0; t < 3; t++) {
      u_out[3 * j + t] = u[t];
      fnx_out[3 * j + t] = fnx[t];
    }
  }
}

void or_window_tensor(const or_plan *p, const double *xj, int interlaced, double *psi, double *dpsi, double *ddpsi) {
  double x[3], fnx[3];
  I64 u[3];
  node_setup(p, xj, interlaced, x, fnx, u);
  tensor_psi(p, x, fnx, psi);
  if (dpsi) tensor_dpsi(p, x, fnx, psi, dpsi);
  if (dpsi && ddpsi) tensor_ddpsi(p, x, fnx, psi, dpsi, ddpsi);
}

static inline I64 wrapi(I64 a, I64 n) {
  I64 r = a % n;
  return r < 0 ? r + n : r;
}

/* ---------------------------------------------------------------------------
 * matrix B: interpolation, ndft-parallel.c:2703-2888 with assign.c:667-1159.
 *   grid: n0*n1*n2 complex (c2c) or real (c2r), natural order
 *   out arrays are complex (c2c) or real (c2r); ind = j*stride + offset
 * ------------------------------------------------------------------------- */
void or_trafo_B(const or_plan *p, I64 M, const double *xall, const void *gridv, double *f, double *grad, double *hess,
                I64 offset, I64 stride, int use_il, int il, unsigned cflags, int nthreads) {
  const int cut = p->cutoff;
  const I64 n0 = p->n[0], n1 = p->n[1], n2 = p->n[2];
  const int c2r = p->c2r;
  /* c2c + PNFFT_PRE_QUAD_PSI (bit 4 == node flag PNFFT_REAL_F) reads only the
   * real parts of the grid, ndft-parallel.c:2804-2842 */
  const int real_only = (!c2r) && (p->flags & F_REAL_F);
  const cplx *gc = (const cplx *)gridv;
  const double *gr = (const double *)gridv;
  const int need_d = (cflags & (C_GRAD | C_HESS)) != 0, need_dd = (cflags & C_HESS) != 0;
  /* nodes are taken in the order of their lowest grid plane in axis 0 (as the
   * reference's PNFFT_SORT_NODES does for cache reuse); every node's sum is
   * independent of the order */
  I64 *order = (I64 *)malloc(sizeof(I64) * (M > 0 ? M : 1));
  {
    I64 *cnt = (I64 *)calloc(n0 + 1, sizeof(I64));
    I64 *pl = (I64 *)malloc(sizeof(I64) * (M > 0 ? M : 1));
    for (I64 j = 0; j < M; j++) {
      double x[3], fnx[3];
      I64 u[3];
      node_setup(p, xall + 3 * j, il, x, fnx, u);
      pl[j] = wrapi(u[0], n0);
      cnt[pl[j] + 1]++;
    }
    for (I64 q = 0; q < n0; q++) cnt[q + 1] += cnt[q];
    for (I64 j = 0; j < M; j++) order[cnt[pl[j]]++] = j;
    free(cnt);
    free(pl);
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
#endif
  for (I64 q = 0; q < M; q++) {
    const I64 j = order[q];
    double x[3], fnx[3], psi[3 * 64], dpsi[3 * 64], ddpsi[3 * 64];
    I64 u[3];
    node_setup(p, xall + 3 * j, il, x, fnx, u);
    tensor_psi(p, x, fnx, psi);
    if (need_d) tensor_dpsi(p, x, fnx, psi, dpsi);
    if (need_dd) tensor_ddpsi(p, x, fnx, psi, dpsi, ddpsi);
    const double *px = psi, *py = psi + cut, *pz = psi + 2 * cut;
    const double *dx = dpsi, *dy = dpsi + cut, *dz = dpsi + 2 * cut;
    const double *ddx = ddpsi, *ddy = ddpsi + cut, *ddz = ddpsi + 2 * cut;
    cplx a_f = 0, a_g[3] = {0, 0, 0}, a_h[6] = {0, 0, 0, 0, 0, 0};
    I64 i2[64];
    for (int l2 = 0; l2 < cut; l2++) i2[l2] = wrapi(u[2] + l2, n2);
    for (int l0 = 0; l0 < cut; l0++) {
      I64 i0 = wrapi(u[0] + l0, n0);
      for (int l1 = 0; l1 < cut; l1++) {
        I64 row = (i0 * n1 + wrapi(u[1] + l1, n1)) * n2;
        double pxy = px[l0] * py[l1];
        double pdxy = 0, pxdy = 0, pdxdy = 0, pddxy = 0, pxddy = 0;
        if (need_d) {
          pdxy = dx[l0] * py[l1];
          pxdy = px[l0] * dy[l1];
        }
        if (need_dd) {
          pdxdy = dx[l0] * dy[l1];
          pddxy = ddx[l0] * py[l1];
          pxddy = px[l0] * ddy[l1];
        }
        for (int l2 = 0; l2 < cut; l2++) {
          cplx g;
          if (c2r) g = gr[row + i2[l2]];
          else if (real_only) g = creal(gc[row + i2[l2]]);
          else g = gc[row + i2[l2]];
          if (cflags & C_F) a_f += pxy * pz[l2] * g;
          if (cflags & C_GRAD) {
            a_g[0] += pdxy * pz[l2] * g;
            a_g[1] += pxdy * pz[l2] * g;
            a_g[2] += pxy * dz[l2] * g;
          }
          if (cflags & C_HESS) {
            a_h[0] += pddxy * pz[l2] * g;
            a_h[1] += pdxdy * pz[l2] * g;
            a_h[2] += pdxy * dz[l2] * g;
            a_h[3] += pxddy * pz[l2] * g;
            a_h[4] += pxdy * dz[l2] * g;
            a_h[5] += pxy * ddz[l2] * g;
          }
        }
      }
    }
    if (use_il) {
      a_f *= 0.5;
      for (int c = 0; c < 3; c++) a_g[c] *= 0.5;
      for (int c = 0; c < 6; c++) a_h[c] *= 0.5;
    }
    I64 ind = j * stride + offset;
    if (c2r) {
      if ((cflags & C_F) && f) f[ind] += creal(a_f);
      if ((cflags & C_GRAD) && grad)
        for (int c = 0; c < 3; c++) grad[3 * ind + c] += creal(a_g[c]);
      if ((cflags & C_HESS) && hess)
        for (int c = 0; c < 6; c++) hess[6 * ind + c] += creal(a_h[c]);
    } else {
      cplx *fc = (cplx *)f, *gcx = (cplx *)grad, *hc = (cplx *)hess;
      if ((cflags & C_F) && f) fc[ind] += a_f;
      if ((cflags & C_GRAD) && grad)
        for (int c = 0; c < 3; c++) gcx[3 * ind + c] += a_g[c];
      if ((cflags & C_HESS) && hess)
        for (int c = 0; c < 6; c++) hc[6 * ind + c] += a_h[c];
    }
  }
  free(order);
}

/* ---------------------------------------------------------------------------
 * matrix B^T: spreading, ndft-parallel.c:2890-3009 with assign.c:478-664.
 * The grid is accumulated (the caller zeroes it, ndft-parallel.c:2629-2635).
 * Parallel version: nodes are grouped by their lowest x0-plane into slabs at
 * least `cutoff` planes thick; even slabs, then odd slabs, run concurrently so
 * that no two threads add to the same grid point.
 * ------------------------------------------------------------------------- */
static void spread_one(const or_plan *p, const double *xj, cplx fj, const cplx *gj, int use_il, int il, unsigned cflags,
                       void *gridv) {
  const int cut = p->cutoff;
  const I64 n0 = p->n[0], n1 = p->n[1], n2 = p->n[2];
  double x[3], fnx[3], psi[3 * 64], dpsi[3 * 64];
  I64 u[3];
  node_setup(p, xj, il, x, fnx, u);
  tensor_psi(p, x, fnx, psi);
  if (cflags & C_GRAD) tensor_dpsi(p, x, fnx, psi, dpsi);
  const double *px = psi, *py = psi + cut, *pz = psi + 2 * cut;
  const double *dx = dpsi, *dy = dpsi + cut, *dz = dpsi + 2 * cut;
  cplx g0 = 0, g1 = 0, g2 = 0;
  if (cflags & C_GRAD) {
    g0 = gj[0];
    g1 = gj[1];
    g2 = gj[2];
  }
  if (use_il) {
    fj *= 0.5;
    g0 *= 0.5;
    g1 *= 0.5;
    g2 *= 0.5;
  }
  I64 i2[64];
  for (int l2 = 0; l2 < cut; l2++) i2[l2] = wrapi(u[2] + l2, n2);
  cplx *gc = (cplx *)gridv;
  double *gr = (double *)gridv;
  for (int l0 = 0; l0 < cut; l0++) {
    I64 i0 = wrapi(u[0] + l0, n0);
    for (int l1 = 0; l1 < cut; l1++) {
      I64 row = (i0 * n1 + wrapi(u[1] + l1, n1)) * n2;
      double pxy = px[l0] * py[l1];
      double pdxy = 0, pxdy = 0;
      if (cflags & C_GRAD) {
        pdxy = dx[l0] * py[l1];
        pxdy = px[l0] * dy[l1];
      }
      for (int l2 = 0; l2 < cut; l2++) {
        cplx add = 0;
        if (cflags & C_F) add += pxy * pz[l2] * fj;
        if (cflags & C_GRAD) {
          /* the three terms are added one after another, assign.c:580-582 */
          if (p->c2r) {
            gr[row + i2[l2]] += creal(add);
            gr[row + i2[l2]] += creal(pdxy * pz[l2] * g0);
            gr[row + i2[l2]] += creal(pxdy * pz[l2] * g1);
            gr[row + i2[l2]] += creal(pxy * dz[l2] * g2);
          } else {
            gc[row + i2[l2]] += add;
            gc[row + i2[l2]] += pdxy * pz[l2] * g0;
            gc[row + i2[l2]] += pxdy * pz[l2] * g1;
            gc[row + i2[l2]] += pxy * dz[l2] * g2;
          }
        } else {
          if (p->c2r) gr[row + i2[l2]] += creal(add);
          else gc[row + i2[l2]] += add;
        }
      }
    }
  }
}

void or_adjoint_B(const or_plan *p, I64 M, const double *xall, const double *f, const double *grad, I64 offset, I64 stride,
                  int use_il, int il, unsigned cflags, void *gridv, int nthreads) {
  const I64 n0 = p->n[0], n1 = p->n[1];
  const int cut = p->cutoff;
  /* blocks of at least `cut` planes in axes 0 and 1; blocks of one colour
   * (parities of both block indices) never touch the same grid points, so a
   * colour's blocks run in parallel and the colours one after another */
  I64 ns0 = n0 / cut, ns1 = n1 / cut;
  if (ns0 % 2) ns0--;
  if (ns1 % 2) ns1--;
  if (ns1 < 2) ns1 = 1;
  const I64 nblk = ns0 * ns1;
  if (nthreads == 1 || ns0 < 2) {
    for (I64 j = 0; j < M; j++) {
      I64 ind = j * stride + offset;
      cplx fj = 0, gj[3] = {0, 0, 0};
      if (p->c2r) {
        if ((cflags & C_F) && f) fj = f[ind];
        if ((cflags & C_GRAD) && grad)
          for (int c = 0; c < 3; c++) gj[c] = grad[3 * ind + c];
      } else {
        if ((cflags & C_F) && f) fj = ((const cplx *)f)[ind];
        if ((cflags & C_GRAD) && grad)
          for (int c = 0; c < 3; c++) gj[c] = ((const cplx *)grad)[3 * ind + c];
      }
      spread_one(p, xall + 3 * j, fj, gj, use_il, il, cflags, gridv);
    }
    return;
  }
  /* bucket nodes by the block of their lowest (x0, x1) grid planes */
  I64 *cnt = (I64 *)calloc(nblk + 1, sizeof(I64));
  I64 *blk = (I64 *)malloc(sizeof(I64) * (M > 0 ? M : 1));
  for (I64 j = 0; j < M; j++) {
    double x[3], fnx[3];
    I64 u[3];
    node_setup(p, xall + 3 * j, il, x, fnx, u);
    I64 b0 = (wrapi(u[0], n0) * ns0) / n0;
    I64 b1 = ns1 > 1 ? (wrapi(u[1], n1) * ns1) / n1 : 0;
    blk[j] = b0 * ns1 + b1;
    cnt[blk[j] + 1]++;
  }
  for (I64 b = 0; b < nblk; b++) cnt[b + 1] += cnt[b];
  I64 *pos = (I64 *)malloc(sizeof(I64) * (nblk + 1));
  memcpy(pos, cnt, sizeof(I64) * (nblk + 1));
  I64 *order = (I64 *)malloc(sizeof(I64) * (M > 0 ? M : 1));
  for (I64 j = 0; j < M; j++) order[pos[blk[j]]++] = j;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  const int ncol1 = ns1 > 1 ? 2 : 1;
  for (int colour = 0; colour < 2 * ncol1; colour++) {
    const I64 p0 = colour / ncol1, p1 = colour % ncol1;
    const I64 h0 = (ns0 - p0 + 1) / 2, h1 = ns1 > 1 ? (ns1 - p1 + 1) / 2 : 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (I64 t = 0; t < h0 * h1; t++) {
      const I64 b = (p0 + 2 * (t / h1)) * ns1 + (ns1 > 1 ? p1 + 2 * (t % h1) : 0);
      for (I64 q = cnt[b]; q < cnt[b + 1]; q++) {
        I64 j = order[q];
        I64 ind = j * stride + offset;
        cplx fj = 0, gj[3] = {0, 0, 0};
        if (p->c2r) {
          if ((cflags & C_F) && f) fj = f[ind];
          if ((cflags & C_GRAD) && grad)
            for (int c = 0; c < 3; c++) gj[c] = grad[3 * ind + c];
        } else {
          if ((cflags & C_F) && f) fj = ((const cplx *)f)[ind];
          if ((cflags & C_GRAD) && grad)
            for (int c = 0; c < 3; c++) gj[c] = ((const cplx *)grad)[3 * ind + c];
        }
        spread_one(p, xall + 3 * j, fj, gj, use_il, il, cflags, gridv);
      }
    }
  }
  free(cnt);
  free(blk);
  free(pos);
  free(order);
}

/* ---------------------------------------------------------------------------
 * matrix D on the N-cube, kernel/matrix_D.c:227-451.  f_hat / g layout:
 * N0 x N1 x N2 row-major, or N1 x N2 x N0 with PNFFT_TRANSPOSED_F_HAT.
 * `Nloc` / `kstart` describe the stored block (c2r stores k2 in [-N2/2, 0]).
 * ------------------------------------------------------------------------- */
static void d_factor_axes(const or_plan *p, const I64 *Nl, const I64 *ks, double *ax[3]) {
  for (int t = 0; t < 3; t++)
    for (I64 k = 0; k < Nl[t]; k++) ax[t][k] = or_inv_phi_hat(p, t, ks[t] + k);
}

/* trafo: out = in * prod inv_phi_hat (overwrite), then the interlacing phase */
void or_trafo_D(const or_plan *p, const I64 *Nl, const I64 *ks, const cplx *in, int interlaced, cplx *out) {
  double *ax[3];
  for (int t = 0; t < 3; t++) ax[t] = (double *)malloc(sizeof(double) * Nl[t]);
  d_factor_axes(p, Nl, ks, ax);
  I64 k = 0;
  if (p->flags & F_TRANSPOSED) {
    for (I64 a1 = 0; a1 < Nl[1]; a1++)
      for (I64 a2 = 0; a2 < Nl[2]; a2++) {
        cplx w12 = ax[1][a1] * ax[2][a2];
        for (I64 a0 = 0; a0 < Nl[0]; a0++, k++) {
          cplx w = w12 * ax[0][a0];
          out[k] = in[k] * w;
        }
      }
  } else {
    for (I64 a0 = 0; a0 < Nl[0]; a0++)
      for (I64 a1 = 0; a1 < Nl[1]; a1++) {
        cplx w01 = ax[0][a0] * ax[1][a1];
        for (I64 a2 = 0; a2 < Nl[2]; a2++, k++) {
          cplx w = w01 * ax[2][a2];
          out[k] = in[k] * w;
        }
      }
  }
  if (interlaced) { /* 282-317, sign = FFTW_FORWARD = -1: factor exp(+pi i h) */
    k = 0;
    if (p->flags & F_TRANSPOSED) {
      for (I64 a1 = 0; a1 < Nl[1]; a1++) {
        double h1 = (double)(ks[1] + a1) / p->n[1];
        for (I64 a2 = 0; a2 < Nl[2]; a2++) {
          double h2 = h1 + (double)(ks[2] + a2) / p->n[2];
          for (I64 a0 = 0; a0 < Nl[0]; a0++, k++) {
            double h0 = h2 + (double)(ks[0] + a0) / p->n[0];
            out[k] *= cexp(PI * I * h0);
          }
        }
      }
    } else {
      for (I64 a0 = 0; a0 < Nl[0]; a0++) {
        double h0 = (double)(ks[0] + a0) / p->n[0];
        for (I64 a1 = 0; a1 < Nl[1]; a1++) {
          double h1 = h0 + (double)(ks[1] + a1) / p->n[1];
          for (I64 a2 = 0; a2 < Nl[2]; a2++, k++) {
            double h2 = h1 + (double)(ks[2] + a2) / p->n[2];
            out[k] *= cexp(PI * I * h2);
          }
        }
      }
    }
  }
  for (int t = 0; t < 3; t++) free(ax[t]);
}

/* adjoint: interlacing phase on g (in place), then out += g * prod inv_phi_hat */
void or_adjoint_D(const or_plan *p, const I64 *Nl, const I64 *ks, cplx *g, int interlaced, cplx *out) {
  I64 k = 0;
  if (interlaced) { /* sign = FFTW_BACKWARD = +1: factor exp(-pi i h) */
    if (p->flags & F_TRANSPOSED) {
      for (I64 a1 = 0; a1 < Nl[1]; a1++) {
        double h1 = (double)(ks[1] + a1) / p->n[1];
        for (I64 a2 = 0; a2 < Nl[2]; a2++) {
          double h2 = h1 + (double)(ks[2] + a2) / p->n[2];
          for (I64 a0 = 0; a0 < Nl[0]; a0++, k++) {
            double h0 = h2 + (double)(ks[0] + a0) / p->n[0];
            g[k] *= cexp(-PI * I * h0);
          }
        }
      }
    } else {
      for (I64 a0 = 0; a0 < Nl[0]; a0++) {
        double h0 = (double)(ks[0] + a0) / p->n[0];
        for (I64 a1 = 0; a1 < Nl[1]; a1++) {
          double h1 = h0 + (double)(ks[1] + a1) / p->n[1];
          for (I64 a2 = 0; a2 < Nl[2]; a2++, k++) {
            double h2 = h1 + (double)(ks[2] + a2) / p->n[2];
            g[k] *= cexp(-PI * I * h2);
          }
        }
      }
    }
  }
  double *ax[3];
  for (int t = 0; t < 3; t++) ax[t] = (double *)malloc(sizeof(double) * Nl[t]);
  d_factor_axes(p, Nl, ks, ax);
  k = 0;
  if (p->flags & F_TRANSPOSED) {
    for (I64 a1 = 0; a1 < Nl[1]; a1++)
      for (I64 a2 = 0; a2 < Nl[2]; a2++) {
        cplx w12 = ax[1][a1] * ax[2][a2];
        for (I64 a0 = 0; a0 < Nl[0]; a0++, k++) out[k] += g[k] * (w12 * ax[0][a0]);
      }
  } else {
    for (I64 a0 = 0; a0 < Nl[0]; a0++)
      for (I64 a1 = 0; a1 < Nl[1]; a1++) {
        cplx w01 = ax[0][a0] * ax[1][a1];
        for (I64 a2 = 0; a2 < Nl[2]; a2++, k++) out[k] += g[k] * (w01 * ax[2][a2]);
      }
  }
  for (int t = 0; t < 3; t++) free(ax[t]);
}

/* ik differentiation scalings on the N-cube, ndft-parallel.c:3012-3087 */
static void ik_loop_index(const or_plan *p, const I64 *Nl, const I64 *ks, I64 k, I64 *kk) {
  if (p->flags & F_TRANSPOSED) { /* N1 x N2 x N0 */
    I64 a0 = k % Nl[0], r = k / Nl[0];
    I64 a2 = r % Nl[2], a1 = r / Nl[2];
    kk[0] = ks[0] + a0;
    kk[1] = ks[1] + a1;
    kk[2] = ks[2] + a2;
  } else {
    I64 a2 = k % Nl[2], r = k / Nl[2];
    I64 a1 = r % Nl[1], a0 = r / Nl[1];
    kk[0] = ks[0] + a0;
    kk[1] = ks[1] + a1;
    kk[2] = ks[2] + a2;
  }
}
void or_trafo_scale_ik(const or_plan *p, const I64 *Nl, const I64 *ks, const cplx *buf, int dim, cplx *g) {
  I64 tot = Nl[0] * Nl[1] * Nl[2];
  for (I64 k = 0; k < tot; k++) {
    I64 kk[3];
    ik_loop_index(p, Nl, ks, k, kk);
    g[k] = -2 * PI * I * kk[dim] * buf[k];
  }
}
void or_trafo_scale_ik2(const or_plan *p, const I64 *Nl, const I64 *ks, const cplx *buf, int dim, cplx *g) {
  static const int T1[6] = {0, 0, 0, 1, 1, 2}, T2[6] = {0, 1, 2, 1, 2, 2};
  double c = -4.0 * PI * PI;
  I64 tot = Nl[0] * Nl[1] * Nl[2];
  for (I64 k = 0; k < tot; k++) {
    I64 kk[3];
    ik_loop_index(p, Nl, ks, k, kk);
    g[k] = c * kk[T1[dim]] * kk[T2[dim]] * buf[k];
  }
}
void or_adjoint_scale_ik(const or_plan *p, const I64 *Nl, const I64 *ks, const cplx *g, int dim, cplx *buf) {
  I64 tot = Nl[0] * Nl[1] * Nl[2];
  for (I64 k = 0; k < tot; k++) {
    I64 kk[3];
    ik_loop_index(p, Nl, ks, k, kk);
    buf[k] += 2 * PI * I * kk[dim] * g[k];
  }
}

/* ---------------------------------------------------------------------------
 * direct NDFT, ndft-parallel.c:356-722 (one block covers all of f_hat)
 * ------------------------------------------------------------------------- */
static int is_hermitian(I64 k0, I64 k1, I64 k2, I64 N0, I64 N1, I64 N2) { /* 356-374 */
  if ((k0 == 0 || k0 == -N0 / 2) && (k1 == 0 || k1 == -N1 / 2) && (k2 == 0 || k2 == -N2 / 2)) return 1;
  if (k1 > 0 && (k2 == 0 || k2 == -N2 / 2)) return 1;
  if (k0 > 0 && (k1 == 0 || k1 == -N1 / 2) && (k2 == 0 || k2 == -N2 / 2)) return 1;
  return 0;
}

void or_ndft_trafo(const or_plan *p, const I64 *Nl, const I64 *ks, I64 M, const double *x, const cplx *fhat, double *f,
                   double *grad, double *hess, unsigned cflags, int nthreads) {
  const int tr = (p->flags & F_TRANSPOSED) != 0;
  const int t0 = tr ? 1 : 0, t1 = tr ? 2 : 1, t2 = tr ? 0 : 2; /* 431-440 */
  const int s[6] = {tr ? 3 : 0, tr ? 4 : 1, tr ? 1 : 2, tr ? 5 : 3, tr ? 2 : 4, tr ? 0 : 5};
  const int c2r = p->c2r;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (I64 j = 0; j < M; j++) {
    cplx ex0 = cexp(-2.0 * PI * x[3 * j + t0] * I), ex1 = cexp(-2.0 * PI * x[3 * j + t1] * I),
         ex2 = cexp(-2.0 * PI * x[3 * j + t2] * I);
    cplx es0 = cexp(-2.0 * PI * ks[t0] * x[3 * j + t0] * I), es1 = cexp(-2.0 * PI * ks[t1] * x[3 * j + t1] * I),
         es2 = cexp(-2.0 * PI * ks[t2] * x[3 * j + t2] * I);
    double fr = 0, gr[3] = {0, 0, 0}, hr[6] = {0, 0, 0, 0, 0, 0};
    cplx fc = 0, gcx[3] = {0, 0, 0}, hc[6] = {0, 0, 0, 0, 0, 0};
    I64 mm = 0;
    cplx e0 = es0;
    for (I64 k0 = ks[t0]; k0 < ks[t0] + Nl[t0]; k0++) {
      cplx e1 = e0 * es1;
      for (I64 k1 = ks[t1]; k1 < ks[t1] + Nl[t1]; k1++) {
        cplx e2 = e1 * es2;
        for (I64 k2 = ks[t2]; k2 < ks[t2] + Nl[t2]; k2++, mm++) {
          cplx bt = fhat[mm] * e2;
          if (c2r) {
            int zero = (k0 == 0 && k1 == 0 && k2 == 0);
            int herm = is_hermitian(k0, k1, k2, p->N[t0], p->N[t1], p->N[t2]);
            if (cflags & C_F) {
              if (zero) fr += creal(fhat[mm]);
              else if (!herm) fr += 2 * creal(bt);
            }
            if (!zero && !herm) {
              if (cflags & C_GRAD) {
                gr[0] += 2 * k0 * cimag(bt);
                gr[1] += 2 * k1 * cimag(bt);
                gr[2] += 2 * k2 * cimag(bt);
              }
              if (cflags & C_HESS) {
                hr[0] += 2 * k0 * k0 * creal(bt);
                hr[1] += 2 * k0 * k1 * creal(bt);
                hr[2] += 2 * k0 * k2 * creal(bt);
                hr[3] += 2 * k1 * k1 * creal(bt);
                hr[4] += 2 * k1 * k2 * creal(bt);
                hr[5] += 2 * k2 * k2 * creal(bt);
              }
            }
          } else {
            if (cflags & C_F) fc += bt;
            if (cflags & C_GRAD) {
              gcx[0] += k0 * bt;
              gcx[1] += k1 * bt;
              gcx[2] += k2 * bt;
            }
            if (cflags & C_HESS) {
              hc[0] += k0 * k0 * bt;
              hc[1] += k0 * k1 * bt;
              hc[2] += k0 * k2 * bt;
              hc[3] += k1 * k1 * bt;
              hc[4] += k1 * k2 * bt;
              hc[5] += k2 * k2 * bt;
            }
          }
          e2 *= ex2;
        }
        e1 *= ex1;
      }
      e0 *= ex0;
    }
    const int tt[3] = {t0, t1, t2};
    const double m2p = -2.0 * PI, m4pp = -4.0 * PI * PI;
    if (c2r) {
      if (cflags & C_F) f[j] += fr;
      if (cflags & C_GRAD)
        for (int c = 0; c < 3; c++) grad[3 * j + tt[c]] += gr[c] * m2p;
      if (cflags & C_HESS)
        for (int c = 0; c < 6; c++) hess[6 * j + s[c]] += hr[c] * m4pp;
    } else {
      cplx *F = (cplx *)f, *G = (cplx *)grad, *H = (cplx *)hess;
      if (cflags & C_F) F[j] += fc;
      if (cflags & C_GRAD)
        for (int c = 0; c < 3; c++) G[3 * j + tt[c]] += gcx[c] * (m2p * I);
      if (cflags & C_HESS)
        for (int c = 0; c < 6; c++) H[6 * j + s[c]] += hc[c] * m4pp;
    }
  }
}

/* adjoint NDFT, 617-722: f_hat[k] += sum_j (f_j + 2 pi i k.grad_j) e^{+2 pi i k x_j} */
void or_ndft_adj(const or_plan *p, const I64 *Nl, const I64 *ks, I64 M, const double *x, const double *f, const double *grad,
                 unsigned cflags, cplx *fhat, int nthreads) {
  const int tr = (p->flags & F_TRANSPOSED) != 0;
  const int t0 = tr ? 1 : 0, t1 = tr ? 2 : 1, t2 = tr ? 0 : 2;
  const int c2r = p->c2r;
  I64 tot = Nl[0] * Nl[1] * Nl[2];
  /* parallel over frequency blocks of the slowest axis, so that every thread
   * owns distinct f_hat entries; per block the node loop runs in order */
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (I64 a0 = 0; a0 < Nl[t0]; a0++) {
    I64 k0 = ks[t0] + a0;
    I64 base = a0 * Nl[t1] * Nl[t2];
    for (I64 j = 0; j < M; j++) {
      cplx ex1 = cexp(+2.0 * PI * x[3 * j + t1] * I), ex2 = cexp(+2.0 * PI * x[3 * j + t2] * I);
      cplx es1 = cexp(+2.0 * PI * ks[t1] * x[3 * j + t1] * I), es2 = cexp(+2.0 * PI * ks[t2] * x[3 * j + t2] * I);
      cplx e0 = cexp(+2.0 * PI * k0 * x[3 * j + t0] * I);
      if (cflags & C_F) {
        cplx fj = c2r ? (cplx)f[j] : ((const cplx *)f)[j];
        cplx e1 = fj * e0 * es1;
        I64 mm = base;
        for (I64 k1 = ks[t1]; k1 < ks[t1] + Nl[t1]; k1++) {
          cplx e2 = e1 * es2;
          for (I64 k2 = ks[t2]; k2 < ks[t2] + Nl[t2]; k2++, mm++) {
            fhat[mm] += e2;
            e2 *= ex2;
          }
          e1 *= ex1;
        }
      }
      if (cflags & C_GRAD) {
        cplx g[3];
        for (int t = 0; t < 3; t++) g[t] = c2r ? (cplx)grad[3 * j + t] : ((const cplx *)grad)[3 * j + t];
        cplx sk0 = g[t0] * (double)k0;
        cplx e1 = 2.0 * PI * I * e0 * es1;
        I64 mm = base;
        for (I64 k1 = ks[t1]; k1 < ks[t1] + Nl[t1]; k1++) {
          cplx sk1 = g[t1] * (double)k1 + sk0;
          cplx e2 = e1 * es2;
          for (I64 k2 = ks[t2]; k2 < ks[t2] + Nl[t2]; k2++, mm++) {
            fhat[mm] += (g[t2] * (double)k2 + sk1) * e2;
            e2 *= ex2;
          }
          e1 *= ex1;
        }
      }
    }
  }
  (void)tot;
}

/* ---------------------------------------------------------------------------
 * node sort of PNFFT_SORT_NODES: keys ((u0 n1 + u1) n2 + u2), u_t =
 * (floor(n_t x_t - m) mod n_t), then a stable LSD radix sort with 9-bit digits
 * over bits [0, ceil(log2(n0 n1 n2)) - 1], ndft-parallel.c:2121-2159 and
 * util/util.c:166-275.  pairs[2p] = key, pairs[2p+1] = original index.
 * ------------------------------------------------------------------------- */
void or_sort_nodes(const or_plan *p, I64 M, const double *x, I64 *pairs) {
  const I64 *n = p->n;
  for (I64 i = 0; i < M; i++) {
    I64 key = 0;
    for (int j = 0; j < 3; j++) {
      I64 h = (I64)floor(n[j] * x[3 * i + j] - p->m);
      I64 uj = (h % n[j] + n[j]) % n[j];
      key += uj;
      if (j + 1 < 3) key *= n[j + 1];
    }
    pairs[2 * i] = key;
    pairs[2 * i + 1] = i;
  }
  double nprod = (double)n[0] * (double)n[1] * (double)n[2];
  I64 rhigh = (I64)ceil(log2(nprod)) - 1;
  I64 *tmp = (I64 *)malloc(sizeof(I64) * 2 * (M > 0 ? M : 1));
  I64 *from = pairs, *to = tmp;
  const I64 rw = 9, rn = 1 << 9, mask = rn - 1;
  I64 shift = 0;
  I64 cnt[512];
  while (rhigh >= 0) {
    memset(cnt, 0, sizeof(cnt));
    for (I64 i = 0; i < M; i++) cnt[(from[2 * i] >> shift) & mask]++;
    I64 acc = 0;
    for (I64 d = 0; d < rn; d++) {
      I64 c = cnt[d];
      cnt[d] = acc;
      acc += c;
    }
    for (I64 i = 0; i < M; i++) {
      I64 d = (from[2 * i] >> shift) & mask;
      to[2 * cnt[d]] = from[2 * i];
      to[2 * cnt[d] + 1] = from[2 * i + 1];
      cnt[d]++;
    }
    I64 *t = from;
    from = to;
    to = t;
    shift += rw;
    rhigh -= rw;
  }
  if (from != pairs) memcpy(pairs, from, sizeof(I64) * 2 * M);
  free(tmp);
}

/* ---------------------------------------------------------------------------
 * reference input generators (glibc rand): api/api-adv.c:35-86 and
 * api/api-basic.c:681-691
 * ------------------------------------------------------------------------- */
void or_srand(unsigned s) { srand(s); }
static double rand_lt1(void) {
  double t;
  do {
    int it = rand();
    t = (double)it / RAND_MAX;
  } while (t >= 1.0);
  return t;
}
void or_init_x_3d_adv(const double *lo, const double *up, const double *x_max, I64 M, double *x) {
  for (int t = 0; t < 3; t++)
    if (lo[t] < -x_max[t] || x_max[t] < up[t]) return;
  for (I64 j = 0; j < M; j++)
    for (int t = 0; t < 3; t++) {
      double v;
      do {
        v = rand_lt1();
        v = (up[t] - lo[t]) * v + lo[t];
      } while (v < -x_max[t] || x_max[t] <= v);
      x[3 * j + t] = v;
    }
}
void or_init_f(I64 M, double *data) {
  for (I64 j = 0; j < M; j++) {
    double re = 100.0 * (double)rand() / RAND_MAX;
    double im = 100.0 * (double)rand() / RAND_MAX;
    data[2 * j] = re;
    data[2 * j + 1] = im;
  }
}
/* The adjoint NDFT of ndft-parallel.c:617-722 (f_hat[k] += f_j e^{+2 pi i k.x_j},
 * c2c, f only) evaluated at the frequencies of a lattice k = (k0[i0], k1[i1],
 * k2[i2]) instead of at all of them, summed over all M nodes.  Each node's
 * factor is formed from one direct cexp per axis and frequency (no
 * recurrence), so the FP64 values stay within a few ulps of the terms'.  Node
 * chunks are summed by the threads in private lattices that are added in
 * thread order.  out has n0*n1*n2 entries, i2 fastest. */
void or_ndft_adj_lattice(I64 M, const double *x, const double *f, int n0, const I64 *k0, int n1, const I64 *k1,
                         int n2, const I64 *k2, cplx *out, int nthreads) {
  const I64 L = (I64)n0 * n1 * n2;
  for (I64 i = 0; i < L; i++) out[i] = 0;
  int nt = 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  nt = omp_get_max_threads();
#endif
  double *acc = (double *)calloc((size_t)nt * 2 * L, sizeof(double));
  if (!acc) return;
#ifdef _OPENMP
#pragma omp parallel
#endif
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double *a = acc + (size_t)tid * 2 * L;
    double *e = (double *)malloc(sizeof(double) * 2 * (size_t)(n0 + n1 + n2));
    double *e0 = e, *e1 = e + 2 * n0, *e2 = e + 2 * (n0 + n1);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (I64 j = 0; j < M; j++) {
      const double fr = f[2 * j], fi = f[2 * j + 1];
      for (int i = 0; i < n0; i++) {
        cplx v = cexp(+2.0 * PI * (double)k0[i] * x[3 * j] * I);
        /* f_j e0 */
        e0[2 * i] = fr * creal(v) - fi * cimag(v);
        e0[2 * i + 1] = fr * cimag(v) + fi * creal(v);
      }
      for (int i = 0; i < n1; i++) {
        cplx v = cexp(+2.0 * PI * (double)k1[i] * x[3 * j + 1] * I);
        e1[2 * i] = creal(v);
        e1[2 * i + 1] = cimag(v);
      }
      for (int i = 0; i < n2; i++) {
        cplx v = cexp(+2.0 * PI * (double)k2[i] * x[3 * j + 2] * I);
        e2[2 * i] = creal(v);
        e2[2 * i + 1] = cimag(v);
      }
      double *o = a;
      for (int i0 = 0; i0 < n0; i0++)
        for (int i1 = 0; i1 < n1; i1++) {
          const double br = e0[2 * i0] * e1[2 * i1] - e0[2 * i0 + 1] * e1[2 * i1 + 1];
          const double bi = e0[2 * i0] * e1[2 * i1 + 1] + e0[2 * i0 + 1] * e1[2 * i1];
          for (int i2 = 0; i2 < n2; i2++, o += 2) {
            o[0] += br * e2[2 * i2] - bi * e2[2 * i2 + 1];
            o[1] += br * e2[2 * i2 + 1] + bi * e2[2 * i2];
          }
        }
    }
    free(e);
  }
  for (int t = 0; t < nt; t++)
    for (I64 i = 0; i < L; i++) out[i] += acc[(size_t)t * 2 * L + 2 * i] + acc[(size_t)t * 2 * L + 2 * i + 1] * I;
  free(acc);
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
