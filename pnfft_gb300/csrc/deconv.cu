// deconv.cu -- the deconvolution D with the zero-padding/cropping that PFFT
// performs around the oversampled FFT, fused into one pass each way.
//
// trafo  (kernel/matrix_D.c:227-252, 319-356; the N -> n zero padding of the
//        forward PFFT plan, ndft-parallel.c:963-974):
//   grid[k mod n] = f_hat[k] * prod_t inv_phi_hat_t(k_t)
//                   (* exp(+pi i sum_t k_t/n_t) on the interlaced pass, 282-317)
//                   (* -2 pi i k_d, or -4 pi^2 k_a k_b, for ik derivatives,
//                      ndft-parallel.c:3034-3087)
//   and zero on every other grid point -- the whole n0 x n1 x n2 grid is
//   written once, coalesced, in natural FFT order.
// adjoint (matrix_D.c:255-280, 358-395; ndft-parallel.c:3012-3032):
//   f_hat[k] += grid[k mod n] (* exp(-pi i sum k_t/n_t)) (* 2 pi i k_d)
//               * prod_t inv_phi_hat_t(k_t)
// c2r plans store the half spectrum k2 in [-N2/2, 0]; the forward pass turns
// it into the c2c spectrum whose real part is the c2r result (weight 2 on the
// non-redundant coefficients, 1 on the real part of k = 0, 0 on the redundant
// ones of is_hermitian, ndft-parallel.c:356-374).
// The products use FP64 (the window coefficients are FP64 tables); the grid
// element is float2 or double2.
#include <cuda_runtime.h>

#include <algorithm>

#include "pg_kernels.h"

namespace pg {

__device__ __forceinline__ bool is_redundant(long long k0, long long k1, long long k2, int N0, int N1, int N2) {
  bool e0 = (k0 == 0 || k0 == -N0 / 2), e1 = (k1 == 0 || k1 == -N1 / 2), e2 = (k2 == 0 || k2 == -N2 / 2);
  if (e0 && e1 && e2) return true;
  if (k1 > 0 && e2) return true;
  if (k0 > 0 && e1 && e2) return true;
  return false;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// ik factor for frequency k: gradient -2 pi i k_d (trafo) / +2 pi i k_d (adjoint),
// Hessian -4 pi^2 k_a k_b
__device__ __forceinline__ double2 ik_factor(const DeconvArgs &a, const long long *k, bool adjoint) {
  const double pi = 3.14159265358979323846;
  if (a.ik == 1) {
    double v = (adjoint ? 2.0 : -2.0) * pi * (double)k[a.ik_dim];
    return make_double2(0.0, v);
  }
  if (a.ik == 2) {
    const int t1[6] = {0, 0, 0, 1, 1, 2}, t2[6] = {0, 1, 2, 1, 2, 2};
    return make_double2(-4.0 * pi * pi * (double)k[t1[a.ik_dim]] * (double)k[t2[a.ik_dim]], 0.0);
  }
  return make_double2(1.0, 0.0);
}

// position of frequency k in the stored f_hat block
__device__ __forceinline__ int64_t fhat_index(const DeconvArgs &a, const long long *k) {
  int64_t a0 = k[0] - a.ks[0], a1 = k[1] - a.ks[1], a2 = k[2] - a.ks[2];
  if (a.transposed) return (a1 * a.Nl[2] + a2) * a.Nl[0] + a0;  // N1 x N2 x N0
  return (a0 * a.Nl[1] + a1) * a.Nl[2] + a2;
}

template <typename C>
__device__ __forceinline__ C to_c(double2 v);
template <>
__device__ __forceinline__ float2 to_c<float2>(double2 v) {
  return make_float2((float)v.x, (float)v.y);
}
template <>
__device__ __forceinline__ double2 to_c<double2>(double2 v) {
  return v;
}
__device__ __forceinline__ double2 to_d(float2 v) { return make_double2((double)v.x, (double)v.y); }
__device__ __forceinline__ double2 to_d(double2 v) { return v; }

template <typename C>
__global__ void k_deconv_pad(DeconvArgs a) {
  const int64_t n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
  const int64_t total = n0 * n1 * n2;
  C *grid = (C *)a.grid;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t i2 = idx % n2, r = idx / n2;
    int64_t i1 = r % n1, i0 = r / n1;
    const int64_t ii[3] = {i0, i1, i2};
    long long k[3];
    bool inside = true;
    for (int t = 0; t < 3; t++) {
      int64_t nt = a.n[t];
      // frequency of this FFT bin: the k = ii (mod n) inside the stored
      // range [ks, ks + Nl) if any (for odd n, bin (n-1)/2 is +(n-1)/2)
      long long kk = (ii[t] < a.ks[t] + a.Nl[t]) ? ii[t] : ii[t] - nt;
      if (kk < a.ks[t] || kk >= a.ks[t] + a.Nl[t]) inside = false;
      k[t] = kk;
    }
    double2 v = make_double2(0.0, 0.0);
    if (inside) {
      const double2 *fh = (const double2 *)a.fhat_in;
      double2 f = fh[fhat_index(a, k)];
      double w = (a.inv[0][k[0] - a.ks[0]] * a.inv[1][k[1] - a.ks[1]]) * a.inv[2][k[2] - a.ks[2]] * a.scale;
      v = make_double2(f.x * w, f.y * w);
      if (a.interlaced) {
        double h = ((double)k[0] / (double)a.n[0] + (double)k[1] / (double)a.n[1]) + (double)k[2] / (double)a.n[2];
        double sn, cs;
        sincospi(h, &sn, &cs);
        v = cmul(v, make_double2(cs, sn));
      }
      if (a.ik) v = cmul(v, ik_factor(a, k, false));
      if (a.c2r) {
        if (k[0] == 0 && k[1] == 0 && k[2] == 0) v.y = 0.0;
        else if (is_redundant(k[0], k[1], k[2], a.N[0], a.N[1], a.N[2])) v = make_double2(0.0, 0.0);
        else v = make_double2(2.0 * v.x, 2.0 * v.y);
      }
    }
    grid[idx] = to_c<C>(v);
  }
}

// One CTA per row of the stored f_hat block (grid-stride), threads along its
// fastest axis (k2, or k0 for TRANSPOSED_F_HAT): f_hat[k] += D grid[k mod n].
template <typename C>
__global__ void k_deconv_crop_acc(DeconvArgs a) {
  const C *grid = (const C *)a.grid;
  double2 *fh = (double2 *)a.fhat_out;
  // storage axes, outer to inner
  const int o0 = a.transposed ? 1 : 0, o1 = a.transposed ? 2 : 1, o2 = a.transposed ? 0 : 2;
  const int64_t rows = a.Nl[o0] * a.Nl[o1], len = a.Nl[o2];
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const int64_t ra = r / a.Nl[o1], rb = r - ra * a.Nl[o1];
    for (int64_t c = threadIdx.x; c < len; c += blockDim.x) {
      int64_t ax[3];
      ax[o0] = ra;
      ax[o1] = rb;
      ax[o2] = c;
      const long long k[3] = {a.ks[0] + ax[0], a.ks[1] + ax[1], a.ks[2] + ax[2]};
      int64_t g[3];  // k mod n; |k| <= N/2 <= n/2
      for (int t = 0; t < 3; t++) g[t] = k[t] < 0 ? k[t] + a.n[t] : k[t];
      double2 v = to_d(grid[(g[0] * a.n[1] + g[1]) * a.n[2] + g[2]]);
      if (a.ik) v = cmul(v, ik_factor(a, k, true));
      if (a.interlaced) {
        double h = ((double)k[0] / (double)a.n[0] + (double)k[1] / (double)a.n[1]) + (double)k[2] / (double)a.n[2];
        double sn, cs;
        sincospi(h, &sn, &cs);
        v = cmul(v, make_double2(cs, -sn));
      }
      const double w = (a.inv[0][ax[0]] * a.inv[1][ax[1]]) * a.inv[2][ax[2]] * a.scale;
      const int64_t idx = r * len + c;
      double2 o = fh[idx];
      o.x += v.x * w;
      o.y += v.y * w;
      fh[idx] = o;
    }
  }
}

static int row_threads(int64_t len) { return len >= 256 ? 256 : (len >= 128 ? 128 : 64); }

// grid-stride passes: 64 resident blocks' worth per SM of the current device
static int64_t max_blocks() {
  static int sms[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152 * 64;
  if (!sms[dev] && cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 152 * 64;
  }
  return (int64_t)sms[dev] * 64;
}

void launch_deconv_pad(const DeconvArgs &a, bool fp32, cudaStream_t s) {
  const int64_t total = (int64_t)a.n[0] * a.n[1] * a.n[2];
  const unsigned bl = (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, max_blocks()));
  if (fp32) k_deconv_pad<float2><<<bl, 256, 0, s>>>(a);
  else k_deconv_pad<double2><<<bl, 256, 0, s>>>(a);
}

void launch_deconv_crop_acc(const DeconvArgs &a, bool fp32, cudaStream_t s) {
  const int o1 = a.transposed ? 2 : 1, o2 = a.transposed ? 0 : 2, o0 = a.transposed ? 1 : 0;
  const int64_t rows = a.Nl[o0] * a.Nl[o1];
  if (rows <= 0 || a.Nl[o2] <= 0) return;
  const int th = row_threads(a.Nl[o2]);
  const unsigned bl = (unsigned)std::min<int64_t>(rows, max_blocks());
  if (fp32) k_deconv_crop_acc<float2><<<bl, th, 0, s>>>(a);
  else k_deconv_crop_acc<double2><<<bl, th, 0, s>>>(a);
}

}  // namespace pg
