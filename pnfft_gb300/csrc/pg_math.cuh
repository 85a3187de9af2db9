// pg_math.cuh -- window functions of the NFFT and the special functions they
// need, written once for host and device and for float and double.
//
// A node x with fractional grid position dist = n x - floor(n x) in [0,1)
// touches the grid points l = floor(n x) - m + s, s = 0..2m.  All windows are
// evaluated at y = n x - l = dist + m - s (signed distance in grid cells).
// Formulas follow kernel/ndft-parallel.c of the reference:
//   Kaiser-Bessel 2241-2285, Bessel-I0 2195-2239, Gaussian 2337-2357 and
//   1678-1714, B-spline 1716-1742/1866-1893/2022-2049, sinc power 2386-2418;
// and the window Fourier coefficients of kernel/matrix_D.c:30-225.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define PG_HD __host__ __device__ __forceinline__
#else
#define PG_HD inline
#endif

namespace pg {

enum WindowKind { WIN_KAISER_BESSEL = 0, WIN_GAUSSIAN = 1, WIN_BSPLINE = 2, WIN_SINC_POWER = 3, WIN_BESSEL_I0 = 4 };

constexpr double kPi = 3.14159265358979323846;

template <typename T>
PG_HD T tpi() {
  return (T)kPi;
}

template <typename T>
PG_HD T teps();
template <>
PG_HD double teps<double>() {
  return 2.220446049250313e-16;
}
template <>
PG_HD float teps<float>() {
  return 1.1920929e-07f;
}

// Modified Bessel functions by their power series (all terms positive):
//   I0(x) = sum_k (x^2/4)^k / (k!)^2,  I1(x) = sum_k (x/2)^(2k+1) / (k! (k+1)!)
// Used for the Bessel-I0 window and, on the host in FP64, for the
// Kaiser-Bessel Fourier coefficients.  (The reference takes both from GSL,
// kernel/bessel_i0.c:375 and bessel_i1.c:570.)
template <typename T>
PG_HD T bessel_i0(T x) {
  T q = (T)0.25 * x * x, term = (T)1, sum = (T)1;
  for (int k = 1; k < 400; k++) {
    term *= q / ((T)k * (T)k);
    sum += term;
    if (term <= teps<T>() * (T)0.25 * sum) break;
  }
  return sum;
}

template <typename T>
PG_HD T bessel_i1(T x) {
  T q = (T)0.25 * x * x, term = (T)0.5 * x, sum = term;
  for (int k = 1; k < 400; k++) {
    term *= q / ((T)k * (T)(k + 1));
    sum += term;
    if (fabs(term) <= teps<T>() * (T)0.25 * fabs(sum)) break;
  }
  return sum;
}

// sin(x)/x with the small-argument branches of kernel/sinc.c:26-53
template <typename T>
PG_HD T sinc(T x) {
  const T e = teps<T>();
  const T es = sqrt(e), es2 = sqrt(es);
  T ax = fabs(x);
  if (ax >= es2) return sin(x) / x;
  T r = (T)1;
  if (ax >= e) {
    T x2 = x * x;
    r -= x2 / (T)6;
    if (ax >= es) r += (x2 * x2) / (T)120;
  }
  return r;
}

// Cardinal B-spline M_p (support (0,p)) at t, by the Cox-de Boor recursion
//   M_k(t) = (t M_{k-1}(t) + (k - t) M_{k-1}(t - 1)) / (k - 1)
// carried out on the p pieces at the fractional part of t.
template <typename T>
PG_HD T bspline(int p, T t) {
  if (p < 1 || !(t > (T)0 && t < (T)p)) return (T)0;
  if ((T)p - t < t) t = (T)p - t;
  T fl = floor(t);
  T phi = t - fl;
  int j = (int)fl;
  T v[40];
  v[0] = (T)1;
  for (int k = 2; k <= p; k++) {
    T prev = (T)0;  // v[i-1] of the previous order
    for (int i = 0; i < k; i++) {
      T cur = (i <= k - 2) ? v[i] : (T)0;
      T tt = phi + (T)i;
      v[i] = (tt * cur + ((T)k - tt) * prev) / (T)(k - 1);
      prev = cur;
    }
  }
  return v[j];
}

// Window values at signed distance y (grid cells) for one axis:
// out[0] = psi, out[1] = d psi / dx, out[2] = d^2 psi / dx^2 (x in [0,1) units),
// computed up to derivative order `nder`.  `s_minus_dist` = s - dist is passed
// separately for the B-spline (argument of M_{2m}).
template <typename T>
PG_HD void window_eval(int kind, int m, T n, T b, T y, T s_minus_dist, int nder, T *out) {
  const T pi = tpi<T>();
  const T mm = (T)m;
  switch (kind) {
    case WIN_GAUSSIAN: {
      T psi = exp(-y * y / b) / sqrt(pi * b);
      out[0] = psi;
      if (nder >= 1) out[1] = (T)-2 * n / b * y * psi;
      if (nder >= 2) out[2] = (T)2 * n * n / b * ((T)2 / b * y * y - (T)1) * psi;
      break;
    }
    case WIN_BSPLINE: {
      T t = s_minus_dist;
      out[0] = bspline<T>(2 * m, t);
      if (nder >= 1) out[1] = -n * (bspline<T>(2 * m - 1, t) - bspline<T>(2 * m - 1, t - (T)1));
      if (nder >= 2)
        out[2] = n * n *
                 (bspline<T>(2 * m - 2, t) - (T)2 * bspline<T>(2 * m - 2, t - (T)1) + bspline<T>(2 * m - 2, t - (T)2));
      break;
    }
    case WIN_SINC_POWER: {
      T psi = pow(sinc<T>(pi * y / b), (T)2 * mm) / b;
      out[0] = psi;
      T yy = pi * y / b;
      T q = pi * n / b;
      T dpsi = (T)0;
      if (nder >= 1) {
        dpsi = (fabs(yy) > teps<T>()) ? (T)2 * mm * pi * n / b * ((T)1 / tan(yy) - (T)1 / yy) * psi : (T)0;
        out[1] = dpsi;
      }
      if (nder >= 2) {
        if (fabs(yy) > teps<T>()) {
          T ty = tan(yy);
          out[2] = (T)2 * mm * pi * n / b * ((T)1 / ty - (T)1 / yy) * dpsi +
                   (T)2 * mm * q * q * ((T)1 / (yy * yy) - (T)1 - (T)1 / (ty * ty)) * psi;
        } else {
          out[2] = (T)-2 * mm * q * q / ((T)3 * b);
        }
      }
      break;
    }
    case WIN_BESSEL_I0: {
      T d = mm * mm - y * y;
      T r = (d < (T)0) ? sqrt(-d) : sqrt(d);
      out[0] = (d < (T)0) ? (T)0 : (T)0.5 * bessel_i0<T>(b * r);
      if (nder >= 1) {
        if (d < (T)0) out[1] = (T)0;
        else if (d > (T)0) out[1] = (T)-0.5 * b * n * y * bessel_i1<T>(b * r) / r;
        else {
          T h = (T)0.5 * b * n;
          out[1] = -h * h * y / n;
        }
      }
      if (nder >= 2) {
        if (d < (T)0) out[2] = (T)0;
        else if (d > (T)0)
          out[2] = (T)0.5 * b * n * n / d * (b * y * y * bessel_i0<T>(b * r) - bessel_i1<T>(b * r) / r * (y * y + mm * mm));
        else {
          T t1 = b * b * mm * n, t2 = b * n;
          out[2] = t1 * t1 / (T)16 - t2 * t2 / (T)4;
        }
      }
      break;
    }
    default: {  // Kaiser-Bessel
      T d = mm * mm - y * y;
      T r = (d < (T)0) ? sqrt(-d) : sqrt(d);
      T br = b * r;
      T psi;
      if (d < (T)0) psi = sin(br) / (pi * r);
      else if (d > (T)0) psi = sinh(br) / (pi * r);
      else psi = b / pi;
      out[0] = psi;
      T dpsi = (T)0;
      if (nder >= 1) {
        if (d < (T)0) dpsi = n * y / d * (psi - b * cos(br) / pi);
        else if (d > (T)0) dpsi = n * y / d * (psi - b * cosh(br) / pi);
        else dpsi = -n * mm * b * b * b / ((T)3 * pi);
        out[1] = dpsi;
      }
      if (nder >= 2) {
        T by = b * y;
        if (d < (T)0)
          out[2] = (T)3 * n * y * dpsi / d + n * n * psi / d * ((T)1 + by * by) - b * n * n / (pi * d) * cos(br);
        else if (d > (T)0)
          out[2] = (T)3 * n * y * dpsi / d + n * n * psi / d * ((T)1 + by * by) - b * n * n / (pi * d) * cosh(br);
        else {
          T bn = b * n, bm = b * mm;
          out[2] = b * bn * bn / ((T)15 * pi) * (bm * bm - (T)5);
        }
      }
      break;
    }
  }
}

// One-dimensional window at position x (units of [0,1)), as PNX(psi/dpsi/ddpsi)
// of ndft-parallel.c:2288-2334.
template <typename T>
PG_HD T window_1d(int kind, int m, T n, T b, T x, int der) {
  T out[3] = {0, 0, 0};
  T y = n * x;
  window_eval<T>(kind, m, n, b, y, (T)m - y, der, out);
  return out[der];
}

// Interpolation of a sampled window, ipnfft.h:457-500 (order 0..3; the table
// holds order+1 samples per (k, s), the first at offset -order/2).
template <typename T>
PG_HD T intpol(int order, const T *tab, T dk) {
  switch (order) {
    case 0:
      return tab[0];
    case 1:
      return tab[0] * ((T)1 - dk) + tab[1] * dk;
    case 2: {
      T c0 = dk + (T)1, c1 = dk, c2 = dk - (T)1;
      return (T)0.5 * tab[0] * c1 * c2 - c0 * tab[1] * c2 + (T)0.5 * c0 * c1 * tab[2];
    }
    default: {
      T c0 = dk + (T)1, c1 = dk, c2 = dk - (T)1, c3 = dk - (T)2;
      return (-tab[0] * c1 * c2 * c3 + (T)3 * c0 * tab[1] * c2 * c3 - (T)3 * c0 * c1 * tab[2] * c3 +
              c0 * c1 * c2 * tab[3]) /
             (T)6;
    }
  }
}

}  // namespace pg
