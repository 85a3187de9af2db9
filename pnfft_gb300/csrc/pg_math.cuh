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

// ---------------------------------------------------------------------------
// FP32 window evaluation with a compensated argument.
//
// In FP32 the window argument y = (m - s) + dist carries a rounding error of
// ~ulp(m) (5e-7 at m = 6), and the windows grow like exp(b sqrt(m^2 - y^2))
// (b m ~ 28 for Kaiser-Bessel at sigma = 2), which turns that error into a
// ~2e-6 relative error of every weight.  Here y = k + d (k integer, 0 <= d < 1)
// is kept as an exact two-float, and m^2 - y^2 = (m^2 - k^2) - d (2k + d),
// sqrt, b*r, y^2/b and pi*y/b are carried as float pairs (TwoSum / TwoProd
// with fmaf), so the exponentials see an argument accurate to ~1e-7 absolute.
// ---------------------------------------------------------------------------
struct WinF {
  float n;             // grid size
  float b, b_lo;       // shape parameter as a float pair
  float ib, ib_lo;     // 1/b
  float pb, pb_lo;     // pi/b
  float gnorm;         // 1/sqrt(pi b) (Gaussian)
  int kscale;          // the values are returned times 2^-kscale (see below)
  float wsc;           // 2^-kscale
};

PG_HD void two_sum_f(float a, float b, float &s, float &e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
PG_HD void two_prod_f(float a, float b, float &p, float &e) {
  p = a * b;
  e = fmaf(a, b, -p);
}

// M_p(j + phi) for integer j and phi in [0,1), Cox-de Boor on the pieces with
// the integer and fractional parts kept apart:
//   M_k(phi+i) = (i M_{k-1}(phi+i) + (k-i) M_{k-1}(phi+i-1) + phi (M_{k-1}(phi+i) - M_{k-1}(phi+i-1))) / (k-1)
PG_HD float bspline_jphi(int p, int j, float phi) {
  if (p < 1 || j < 0 || j >= p || (j == 0 && phi == 0.f)) return 0.f;
  float v[40];
  v[0] = 1.f;
  for (int k = 2; k <= p; k++) {
    float prev = 0.f;
    const float inv = 1.f / (float)(k - 1);
    for (int i = 0; i < k; i++) {
      float cur = (i <= k - 2) ? v[i] : 0.f;
      v[i] = (((float)i * cur + (float)(k - i) * prev) + phi * (cur - prev)) * inv;
      prev = cur;
    }
  }
  return v[j];
}

// I0 and I1 in FP32: power series below x = 12; above it the asymptotic
// expansion I_nu(x) ~ e^x / sqrt(2 pi x) sum_k (-1)^k a_k(nu) / x^k with
// a_k(nu) = prod_{j=1..k} (4 nu^2 - (2j-1)^2) / (k! 8^k) (Abramowitz & Stegun
// 9.7.1), whose terms stay below 1e-8 after nine of them at x >= 12; the
// series would accumulate ~1e-6 relative rounding over its ~20 growing terms.
// Both are returned times 2^-k.
PG_HD void bessel_i01_f(float x, int k, float &i0, float &i1) {
  if (x < 12.f) {
    i0 = ldexpf(bessel_i0<float>(x), -k);
    i1 = ldexpf(bessel_i1<float>(x), -k);
    return;
  }
  const float e = ldexpf(expf(x), -k) / sqrtf(2.f * 3.14159265358979f * x);
  const float ix = 1.f / (8.f * x);
  float t0 = 1.f, t1 = 1.f, s0 = 1.f, s1 = 1.f;
  for (int k = 1; k <= 9; k++) {
    const float q = (float)((2 * k - 1) * (2 * k - 1));
    t0 *= q * ix / (float)k;
    t1 *= (q - 4.f) * ix / (float)k;
    s0 += t0;
    s1 += t1;
  }
  i0 = e * s0;
  i1 = e * s1;
}

// Taylor coefficients about z = 0 (z = b^2 (m^2 - y^2)) of the two radial
// windows, used where the closed-form derivatives cancel (|z| < 9):
//   Kaiser-Bessel  psi = (b/pi) S(z),  S(z) = sinh(sqrt z)/sqrt z = sum z^k / (2k+1)!
//   Bessel-I0      psi = T(z) / 2,     T(z) = I0(sqrt z)        = sum z^k / (4^k k!^2)
// Horner evaluation of f, f' and f'' with ten terms (|z|^10 / 21! < 1e-10).
PG_HD void radial_series(bool kb, float z, float &f0, float &f1, float &f2) {
  constexpr int K = 11;
  float c[K];
  c[0] = 1.f;
#pragma unroll
  for (int k = 1; k < K; k++)
    c[k] = kb ? c[k - 1] / (float)((2 * k) * (2 * k + 1)) : c[k - 1] / (float)(4 * k * k);
  f0 = c[K - 1];
  f1 = (float)(K - 1) * c[K - 1];
  f2 = (float)((K - 1) * (K - 2)) * c[K - 1];
#pragma unroll
  for (int k = K - 2; k >= 0; k--) {
    f0 = fmaf(f0, z, c[k]);
    if (k >= 1) f1 = fmaf(f1, z, (float)k * c[k]);
    if (k >= 2) f2 = fmaf(f2, z, (float)(k * (k - 1)) * c[k]);
  }
}

// h(a) = cot a - 1/a and h'(a) = 1/a^2 - 1 - cot^2 a for the sinc-power window.
// Below |a| = 1, where the closed forms cancel, by the series
//   cot a - 1/a = -sum_{j>=1} 2^(2j) |B_2j| a^(2j-1) / (2j)!
// (B_2j the Bernoulli numbers; ten terms, the last below 3e-10 at |a| = 1).
PG_HD void sinc_h(float a, float &h, float &hp) {
  if (fabsf(a) < 1.f) {
    const float c[10] = {1.f / 3.f,
                         1.f / 45.f,
                         2.f / 945.f,
                         1.f / 4725.f,
                         2.f / 93555.f,
                         1382.f / 638512875.f,
                         4.f / 18243225.f,
                         3617.f / 162820783125.f,
                         87734.f / 38979295480125.f,
                         349222.f / 1531329465290625.f};
    const float a2 = a * a;
    float s = c[9], sp = 19.f * c[9];
#pragma unroll
    for (int j = 8; j >= 0; j--) {
      s = fmaf(s, a2, c[j]);
      sp = fmaf(sp, a2, (float)(2 * j + 1) * c[j]);
    }
    h = -a * s;
    hp = -sp;
  } else {
    const float ct = 1.f / tanf(a);
    h = ct - 1.f / a;
    hp = 1.f / (a * a) - 1.f - ct * ct;
  }
}

// window values at y = k + d, derivative order up to nder (out[0..2]), times
// 2^-c.kscale.  The radial windows reach exp(b m) (~1e13 for Kaiser-Bessel at
// m = 7), so their FP32 products psi_x psi_y psi_z would overflow and the
// deconvolved grid values (~1/phi_hat^3) would be subnormal; the host picks
// kscale ~ log2 psi(0) and multiplies D by the inverse power of two, which
// is exact.  The exponentials are scaled before any derivative factor.
PG_HD void window_eval_f(int kind, int m, const WinF &c, int k, float d, int nder, float *out) {
  const float pi = 3.14159265358979f;
  const float mm = (float)m, n = c.n;
  float post = c.wsc;  // applied at the end unless a branch scales itself
  float yh, yl;
  two_sum_f((float)k, d, yh, yl);
  const float y = yh;  // for the multiplicative factors
  switch (kind) {
    case WIN_GAUSSIAN: {
      // q = y^2 = k^2 + d (2k + d), z = q / b
      float s2, se, pr, pe, qh, ql, zh, zl;
      two_sum_f((float)(2 * k), d, s2, se);
      two_prod_f(d, s2, pr, pe);
      pe += d * se;
      two_sum_f((float)(k * k), pr, qh, ql);
      ql += pe;
      two_prod_f(qh, c.ib, zh, zl);
      zl += qh * c.ib_lo + ql * c.ib;
      const float psi = expf(-zh) * (1.f - zl) * c.gnorm;
      out[0] = psi;
      if (nder >= 1) out[1] = -2.f * n * c.ib * y * psi;
      if (nder >= 2) out[2] = 2.f * n * n * c.ib * (2.f * c.ib * (qh + ql) - 1.f) * psi;
      break;
    }
    case WIN_BSPLINE: {
      // psi = M_2m(s - d), s = m - k
      const int s = m - k;
      int j;
      float phi;
      if (d > 0.f) {
        j = s - 1;
        phi = 1.f - d;
      } else {
        j = s;
        phi = 0.f;
      }
      out[0] = bspline_jphi(2 * m, j, phi);
      if (nder >= 1) out[1] = -n * (bspline_jphi(2 * m - 1, j, phi) - bspline_jphi(2 * m - 1, j - 1, phi));
      if (nder >= 2)
        out[2] = n * n *
                 (bspline_jphi(2 * m - 2, j, phi) - 2.f * bspline_jphi(2 * m - 2, j - 1, phi) +
                  bspline_jphi(2 * m - 2, j - 2, phi));
      break;
    }
    case WIN_SINC_POWER: {
      // a = pi y / b as a pair.  The 2m-th power multiplies the relative
      // error of sinc(a) by 2m, so sinc is taken in FP64 (this window only)
      // and its rounding to float is carried as a first-order correction.
      float ah, al;
      two_prod_f(c.pb, yh, ah, al);
      al += c.pb * yl + c.pb_lo * yh;
      const double ad = (double)ah + (double)al;
      const double scd = sinc<double>(ad);
      const float sc = (float)scd;
      const float corr = (scd != 0.0) ? (float)((scd - (double)sc) / scd) : 0.f;
      const float psi = powf(sc, 2.f * mm) * c.ib * (1.f + 2.f * mm * corr + c.ib_lo / c.ib);
      out[0] = psi;
      if (nder >= 1) {
        // d/dx = 2m (pi n / b) h(a) psi;  d2/dx2 = 2m (pi n / b)^2 (h'(a) + 2m h(a)^2) psi
        float h, hp;
        sinc_h(ah, h, hp);
        const float q = pi * n * c.ib;
        out[1] = 2.f * mm * q * h * psi;
        if (nder >= 2) out[2] = 2.f * mm * q * q * (hp + 2.f * mm * h * h) * psi;
      }
      break;
    }
    default: {  // Kaiser-Bessel and Bessel-I0: D = m^2 - y^2
      float s2, se, pr, pe, Dh, Dl;
      two_sum_f((float)(2 * k), d, s2, se);
      two_prod_f(d, s2, pr, pe);
      pe += d * se;
      two_sum_f((float)(m * m - k * k), -pr, Dh, Dl);
      Dl -= pe;
      const float D = Dh + Dl;
      const bool kb = (kind != WIN_BESSEL_I0);
      const float b2 = c.b * c.b, z = b2 * D;
      if (D == 0.f) {
        // the values the reference assigns at |y| = m (both signs of y)
        if (kb) {
          out[0] = c.b / pi;
          if (nder >= 1) out[1] = -n * mm * c.b * c.b * c.b / (3.f * pi);
          if (nder >= 2) {
            const float bn = c.b * n, bm = c.b * mm;
            out[2] = c.b * bn * bn / (15.f * pi) * (bm * bm - 5.f);
          }
        } else {
          out[0] = 0.5f;
          if (nder >= 1) {
            const float h = 0.5f * c.b * n;
            out[1] = -h * h * y / n;
          }
          if (nder >= 2) {
            const float t1 = c.b * c.b * mm * n, t2 = c.b * n;
            out[2] = t1 * t1 / 16.f - t2 * t2 / 4.f;
          }
        }
      } else if (!kb && D < 0.f) {
        out[0] = 0.f;
        if (nder >= 1) out[1] = 0.f;
        if (nder >= 2) out[2] = 0.f;
      } else if (fabsf(z) < 9.f) {
        // psi = A f(z), dpsi/dx = -2 A n b^2 y f'(z), d2psi/dx2 = A n^2 (4 b^4 y^2 f'' - 2 b^2 f')
        float f0, f1, f2;
        radial_series(kb, z, f0, f1, f2);
        const float A = kb ? c.b / pi : 0.5f;
        out[0] = A * f0;
        if (nder >= 1) out[1] = -2.f * A * n * b2 * y * f1;
        if (nder >= 2) out[2] = A * n * n * b2 * (4.f * b2 * y * y * f2 - 2.f * f1);
      } else if (D > 0.f) {
        const float rh = sqrtf(D);
        const float rl = (fmaf(-rh, rh, Dh) + Dl) / (2.f * rh);
        float xh, xl;
        two_prod_f(c.b, rh, xh, xl);
        xl += c.b * rl + c.b_lo * rh;
        post = 1.f;
        if (kb) {
          // xh >= 3 here
          const float E0 = expf(xh) * (1.f + xl);
          const float E = ldexpf(E0, -c.kscale), Ei = ldexpf(1.f / E0, -c.kscale);
          const float sh = 0.5f * (E - Ei), ch = 0.5f * (E + Ei);
          const float psi = sh / (pi * rh) * (1.f - rl / rh);
          out[0] = psi;
          float dpsi = 0.f;
          if (nder >= 1) {
            dpsi = n * y / D * (psi - c.b * ch / pi);
            out[1] = dpsi;
          }
          if (nder >= 2) {
            const float by = c.b * y;
            out[2] = 3.f * n * y * dpsi / D + n * n * psi / D * (1.f + by * by) - c.b * n * n / (pi * D) * ch;
          }
        } else {
          float i0h, i1h;
          bessel_i01_f(xh, c.kscale, i0h, i1h);
          out[0] = 0.5f * (i0h + i1h * xl);
          const float r = rh + rl;
          const float i1 = i1h + (i0h - i1h / xh) * xl;
          if (nder >= 1) out[1] = -0.5f * c.b * n * y * i1 / r;
          if (nder >= 2) {
            const float yy = y * y;
            out[2] = 0.5f * c.b * n * n / D * (c.b * yy * (i0h + i1h * xl) - i1 / r * (yy + mm * mm));
          }
        }
      } else {  // Kaiser-Bessel continued as sin beyond |y| = m
        const float r = sqrtf(-D), br = c.b * r;
        float sn, cs;
        sincosf(br, &sn, &cs);
        const float psi = sn / (pi * r);
        out[0] = psi;
        float dpsi = 0.f;
        if (nder >= 1) {
          dpsi = n * y / D * (psi - c.b * cs / pi);
          out[1] = dpsi;
        }
        if (nder >= 2) {
          const float by = c.b * y;
          out[2] = 3.f * n * y * dpsi / D + n * n * psi / D * (1.f + by * by) - c.b * n * n / (pi * D) * cs;
        }
      }
      break;
    }
  }
  out[0] *= post;
  if (nder >= 1) out[1] *= post;
  if (nder >= 2) out[2] *= post;
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
