// pg_index.cuh -- node-to-grid index math shared by the binning and the
// verification kernels.
#pragma once
#include <cuda_runtime.h>

namespace pg {

// floor(fl(n x)) and the fraction fl(n x) - floor(fl(n x)) for a double x and
// an integer 1 <= n <= 2^20, where fl() is the IEEE round-to-nearest-even
// product that the reference computes in FP64 (ndft-parallel.c:2165-2174).
// Integer arithmetic only: the exact product n * M_x (<= 73 bits) is rounded
// to 53 bits with ties to even, then split into integer and fraction parts.
__device__ __forceinline__ void nx_exact(double x, int n, long long *fnx, float *frac) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int sign = (int)(bits >> 63);
  int E = (int)((bits >> 52) & 0x7ff);
  unsigned long long Mx = bits & ((1ull << 52) - 1);
  if (E == 0) {
    if (Mx == 0) {
      *fnx = 0;
      *frac = 0.f;
      return;
    }
    E = 1;
  } else {
    Mx |= (1ull << 52);
  }
  const unsigned long long nn = (unsigned long long)n;
  const unsigned long long lo = Mx * nn, hi = __umul64hi(Mx, nn);
  const int L = hi ? 128 - __clzll((long long)hi) : 64 - __clzll((long long)lo);
  int sh = L > 53 ? L - 53 : 0;
  unsigned long long q = lo;
  if (sh > 0) {
    q = (lo >> sh) | (hi << (64 - sh));
    const unsigned long long rem = lo & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (q & 1ull))) q++;
    if (q == (1ull << 53)) {
      q >>= 1;
      sh++;
    }
  }
  const int e2 = sh + E - 1075;  // fl(n x) = (-1)^sign q 2^e2
  if (e2 >= 0) {
    long long v = (long long)(q << e2);
    *fnx = sign ? -v : v;
    *frac = 0.f;
    return;
  }
  const int k = -e2;
  unsigned long long ip, fr;
  if (k >= 64) {
    ip = 0;
    fr = q;
  } else {
    ip = q >> k;
    fr = q & ((1ull << k) - 1);
  }
  // |fl(n x)| < 2^-11 when k >= 64: the whole product is fraction
  if (!sign) {
    *fnx = (long long)ip;
    *frac = ldexpf(__ull2float_rn(fr), -k);
  } else if (fr == 0) {
    *fnx = -(long long)ip;
    *frac = 0.f;
  } else {
    *fnx = -(long long)ip - 1;
    // 1 - fr 2^-k, from the integers while 2^k fits in 64 bits
    *frac = (k >= 64) ? 1.f - ldexpf(__ull2float_rn(fr), -k) : ldexpf(__ull2float_rn((1ull << k) - fr), -k);
  }
}


}  // namespace pg
