// ndft.cu -- the direct NDFT of PNFFT_COMPUTE_DIRECT in FP64 on the device.
//
// Reference: trafo_A / adj_A (kernel/ndft-parallel.c:377-722), for the single
// block of a 1x1x1 mesh.  trafo: one thread per node walks all coefficients
// with the exponential recurrences of the reference (456-491); c2r uses the
// redundancy rule is_hermitian (356-374) and the reference's scalings
// (594-612).  adjoint: one thread per (k0, k1) row of coefficients walks all
// nodes, with one recurrence along k2 per node.
#include <cuda_runtime.h>

#include "pg_kernels.h"

namespace pg {

struct dc {
  double x, y;
};
__device__ __forceinline__ dc dmul(dc a, dc b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ dc dexpi(double t) {  // exp(2 pi i t)
  double s, c;
  sincospi(2.0 * t, &s, &c);
  return {c, s};
}

__device__ __forceinline__ bool ndft_herm(long long k0, long long k1, long long k2, long long N0, long long N1,
                                          long long N2) {
  bool e0 = (k0 == 0 || k0 == -N0 / 2), e1 = (k1 == 0 || k1 == -N1 / 2), e2 = (k2 == 0 || k2 == -N2 / 2);
  if (e0 && e1 && e2) return true;
  if (k1 > 0 && e2) return true;
  if (k0 > 0 && e1 && e2) return true;
  return false;
}

__global__ void k_ndft_trafo(NdftArgs a) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.M) return;
  const int tr = a.transposed;
  const int t0 = tr ? 1 : 0, t1 = tr ? 2 : 1, t2 = tr ? 0 : 2;
  const int s[6] = {tr ? 3 : 0, tr ? 4 : 1, tr ? 1 : 2, tr ? 5 : 3, tr ? 2 : 4, tr ? 0 : 5};
  const double x0 = a.x[3 * j + t0], x1 = a.x[3 * j + t1], x2 = a.x[3 * j + t2];
  const dc ex0 = dexpi(-x0), ex1 = dexpi(-x1), ex2 = dexpi(-x2);
  const dc es0 = dexpi(-(double)a.ks[t0] * x0), es1 = dexpi(-(double)a.ks[t1] * x1), es2 = dexpi(-(double)a.ks[t2] * x2);
  const bool F = a.cflags & 1u, G = a.cflags & 2u, H = a.cflags & 4u;
  const dc *fh = (const dc *)a.fhat;
  double fr = 0, gr[3] = {0, 0, 0}, hr[6] = {0, 0, 0, 0, 0, 0};
  dc fc = {0, 0}, gc[3] = {{0, 0}, {0, 0}, {0, 0}}, hc[6] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
  int64_t mm = 0;
  dc e0 = es0;
  for (long long k0 = a.ks[t0]; k0 < a.ks[t0] + a.Nl[t0]; k0++) {
    dc e1 = dmul(e0, es1);
    for (long long k1 = a.ks[t1]; k1 < a.ks[t1] + a.Nl[t1]; k1++) {
      dc e2 = dmul(e1, es2);
      for (long long k2 = a.ks[t2]; k2 < a.ks[t2] + a.Nl[t2]; k2++, mm++) {
        dc bt = dmul(fh[mm], e2);
        if (a.c2r) {
          bool zero = (k0 == 0 && k1 == 0 && k2 == 0);
          bool herm = ndft_herm(k0, k1, k2, a.N[t0], a.N[t1], a.N[t2]);
          if (F) {
            if (zero) fr += fh[mm].x;
            else if (!herm) fr += 2 * bt.x;
          }
          if (!zero && !herm) {
            if (G) {
              gr[0] += 2 * k0 * bt.y;
              gr[1] += 2 * k1 * bt.y;
              gr[2] += 2 * k2 * bt.y;
            }
            if (H) {
              hr[0] += 2 * k0 * k0 * bt.x;
              hr[1] += 2 * k0 * k1 * bt.x;
              hr[2] += 2 * k0 * k2 * bt.x;
              hr[3] += 2 * k1 * k1 * bt.x;
              hr[4] += 2 * k1 * k2 * bt.x;
              hr[5] += 2 * k2 * k2 * bt.x;
            }
          }
        } else {
          if (F) {
            fc.x += bt.x;
            fc.y += bt.y;
          }
          if (G) {
            double kk[3] = {(double)k0, (double)k1, (double)k2};
            for (int c = 0; c < 3; c++) {
              gc[c].x += kk[c] * bt.x;
              gc[c].y += kk[c] * bt.y;
            }
          }
          if (H) {
            double kk[6] = {(double)(k0 * k0), (double)(k0 * k1), (double)(k0 * k2),
                            (double)(k1 * k1), (double)(k1 * k2), (double)(k2 * k2)};
            for (int c = 0; c < 6; c++) {
              hc[c].x += kk[c] * bt.x;
              hc[c].y += kk[c] * bt.y;
            }
          }
        }
        e2 = dmul(e2, ex2);
      }
      e1 = dmul(e1, ex1);
    }
    e0 = dmul(e0, ex0);
  }
  const double pi = 3.14159265358979323846;
  const int tt[3] = {t0, t1, t2};
  if (a.c2r) {
    if (F) a.f[j] = fr;
    if (G)
      for (int c = 0; c < 3; c++) a.grad[3 * j + tt[c]] = gr[c] * (-2.0 * pi);
    if (H)
      for (int c = 0; c < 6; c++) a.hess[6 * j + s[c]] = hr[c] * (-4.0 * pi * pi);
  } else {
    if (F) {
      a.f[2 * j] = fc.x;
      a.f[2 * j + 1] = fc.y;
    }
    if (G)
      for (int c = 0; c < 3; c++) {  // * (-2 pi i)
        a.grad[2 * (3 * j + tt[c])] = gc[c].y * (2.0 * pi);
        a.grad[2 * (3 * j + tt[c]) + 1] = -gc[c].x * (2.0 * pi);
      }
    if (H)
      for (int c = 0; c < 6; c++) {
        a.hess[2 * (6 * j + s[c])] = hc[c].x * (-4.0 * pi * pi);
        a.hess[2 * (6 * j + s[c]) + 1] = hc[c].y * (-4.0 * pi * pi);
      }
  }
}

// adjoint: thread per (a0, a1) row of f_hat in memory order
__global__ void k_ndft_adj(NdftArgs a) {
  const int tr = a.transposed;
  const int t0 = tr ? 1 : 0, t1 = tr ? 2 : 1, t2 = tr ? 0 : 2;
  int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= a.Nl[t0] * a.Nl[t1]) return;
  const long long k0 = a.ks[t0] + row / a.Nl[t1], k1 = a.ks[t1] + row % a.Nl[t1];
  const int64_t L = a.Nl[t2];
  dc *out = (dc *)a.fhat_out + row * L;
  const bool F = a.cflags & 1u, G = a.cflags & 2u;
  const double pi = 3.14159265358979323846;
  for (int64_t j = 0; j < a.M; j++) {
    const double x0 = a.x[3 * j + t0], x1 = a.x[3 * j + t1], x2 = a.x[3 * j + t2];
    dc e = dexpi((double)k0 * x0 + (double)k1 * x1);
    e = dmul(e, dexpi((double)a.ks[t2] * x2));
    const dc st = dexpi(x2);
    dc fj = {0, 0};
    if (F) fj = a.c2r ? dc{a.f_in[j], 0.0} : dc{a.f_in[2 * j], a.f_in[2 * j + 1]};
    dc g[3] = {{0, 0}, {0, 0}, {0, 0}};
    if (G)
      for (int t = 0; t < 3; t++)
        g[t] = a.c2r ? dc{a.grad_in[3 * j + t], 0.0} : dc{a.grad_in[2 * (3 * j + t)], a.grad_in[2 * (3 * j + t) + 1]};
    // 2 pi i (k . grad): k0/k1 fixed along the row, k2 varies
    dc base = {g[t0].x * (double)k0 + g[t1].x * (double)k1, g[t0].y * (double)k0 + g[t1].y * (double)k1};
    for (int64_t c = 0; c < L; c++) {
      long long k2 = a.ks[t2] + c;
      dc w = fj;
      if (G) {
        dc sk = {base.x + g[t2].x * (double)k2, base.y + g[t2].y * (double)k2};
        w.x += -2.0 * pi * sk.y;
        w.y += 2.0 * pi * sk.x;
      }
      dc v = dmul(w, e);
      out[c].x += v.x;
      out[c].y += v.y;
      e = dmul(e, st);
    }
  }
}

void launch_ndft_trafo(const NdftArgs &a, cudaStream_t s) {
  if (a.M <= 0) return;
  k_ndft_trafo<<<(unsigned)((a.M + 127) / 128), 128, 0, s>>>(a);
}

void launch_ndft_adj(const NdftArgs &a, cudaStream_t s) {
  const int tr = a.transposed;
  const int t0 = tr ? 1 : 0, t1 = tr ? 2 : 1;
  int64_t rows = a.Nl[t0] * a.Nl[t1];
  if (rows <= 0) return;
  k_ndft_adj<<<(unsigned)((rows + 127) / 128), 128, 0, s>>>(a);
}

}  // namespace pg
