// float_io.cu -- the transforms of the single-precision API pnfftf_* on the GPU.
//
// The caller's float arrays are copied to the device as float (half the bytes
// of the double arrays) and widened there; the double plan then runs on device
// arrays (zero-copy mode: no host staging, no host-side conversion), and its
// outputs are rounded to float on the device and copied back.  Each float plan
// owns a stream, set on its double plan, on which the copies, the conversions
// and the transform are ordered; a call returns after its outputs are on the
// host, as pnfftf_trafo / pnfftf_adj of the reference do (api/pnfft.h:287 is
// the float expansion of the double API).
#include <cuda_runtime.h>

#include "api_float.h"
#include "pg_internal.h"

namespace pg {

struct FloatBuf {
  float *d32 = nullptr;
  double *d64 = nullptr;
  size_t cap = 0;
};

struct FloatDev {
  FloatBuf b[4];  // nodes: x, f, grad, hess; plan: f_hat in b[0]
  cudaStream_t stream = nullptr;
  const float *last_x = nullptr;  // nodes: the float x uploaded last
  uint64_t x_ver = 0;             // nodes: the node version of that upload (0: none)
};

void float_dev_free(FloatDev *d) {
  if (!d) return;
  if (d->stream) cudaStreamSynchronize(d->stream);
  for (FloatBuf &b : d->b) {
    if (b.d32) cudaFree(b.d32);
    if (b.d64) cudaFree(b.d64);
  }
  if (d->stream) cudaStreamDestroy(d->stream);
  delete d;
}

namespace {

__global__ void k_widen(const float *__restrict__ s, double *__restrict__ d, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (double)s[i];
}

__global__ void k_narrow(const double *__restrict__ s, float *__restrict__ d, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (float)s[i];
}

int conv_blocks(int64_t n) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
  }
  const int64_t need = (n + 255) / 256;
  return (int)(need < 8LL * sms ? (need > 0 ? need : 1) : 8LL * sms);
}

bool cuda_ok(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  set_error("pnfftf: %s: %s", what, cudaGetErrorString(e));
  return false;
}

bool ensure(FloatBuf &b, size_t n) {
  if (n == 0) n = 1;
  if (b.cap >= n) return true;
  if (b.d32) cudaFree(b.d32);
  if (b.d64) cudaFree(b.d64);
  b.d32 = nullptr;
  b.d64 = nullptr;
  b.cap = 0;
  if (!cuda_ok(cudaMalloc(&b.d32, sizeof(float) * n), "device allocation") ||
      !cuda_ok(cudaMalloc(&b.d64, sizeof(double) * n), "device allocation"))
    return false;
  b.cap = n;
  return true;
}

// host float[n] -> device double[n] (through the float copy)
bool upload(FloatBuf &b, const float *h, size_t n, cudaStream_t s) {
  if (!ensure(b, n)) return false;
  if (n == 0) return true;
  if (!cuda_ok(cudaMemcpyAsync(b.d32, h, sizeof(float) * n, cudaMemcpyHostToDevice, s), "copy to the device"))
    return false;
  k_widen<<<conv_blocks((int64_t)n), 256, 0, s>>>(b.d32, b.d64, (int64_t)n);
  return cuda_ok(cudaGetLastError(), "k_widen launch");
}

// device double[n] -> host float[n]
bool download(FloatBuf &b, float *h, size_t n, cudaStream_t s) {
  if (n == 0) return true;
  k_narrow<<<conv_blocks((int64_t)n), 256, 0, s>>>(b.d64, b.d32, (int64_t)n);
  if (!cuda_ok(cudaGetLastError(), "k_narrow launch")) return false;
  return cuda_ok(cudaMemcpyAsync(h, b.d32, sizeof(float) * n, cudaMemcpyDeviceToHost, s), "copy to the host");
}

// the plan's stream (created on first use and set on the double plan) and
// the device x of the nodes
bool begin(pnfftf_plan ths, pnfftf_nodes nodes, cudaStream_t *s) {
  if (!ths->dev) ths->dev = new FloatDev();
  if (!nodes->dev) nodes->dev = new FloatDev();
  if (!ths->dev->stream) {
    if (!cuda_ok(cudaStreamCreateWithFlags(&ths->dev->stream, cudaStreamNonBlocking), "stream creation"))
      return false;
    if (engine_set_stream(ths->p, ths->dev->stream) != 0) return false;
  }
  *s = ths->dev->stream;
  const size_t M = (size_t)(nodes->M > 0 ? nodes->M : 0);
  if (!nodes->x && M > 0) {
    set_error("pnfftf: the nodes have no x array");
    return false;
  }
  // a new x array means new coordinates (as pnfft_set_x of the double API)
  FloatDev *v = nodes->dev;
  if (v->last_x != nodes->x) nodes->nd->version++;
  v->last_x = nodes->x;
  // fixed nodes (pnfftf_precompute_psi): the device copy of x is reused, as
  // the double API does with host arrays
  if (nodes->nd->fixed && v->x_ver == nodes->nd->version && v->b[0].cap >= 3 * M) return true;
  if (!upload(v->b[0], nodes->x, 3 * M, *s)) return false;
  v->x_ver = nodes->nd->version;
  return true;
}

bool finish(pnfftf_plan ths) {
  return cuda_ok(cudaStreamSynchronize(ths->dev->stream), "stream synchronize");
}

}  // namespace
}  // namespace pg

using namespace pg;

int pnfftf_gb300_trafo_dev(pnfftf_plan ths, pnfftf_nodes nodes, unsigned cflags) {
  cudaStream_t s;
  if (!begin(ths, nodes, &s)) return -1;
  const size_t M = (size_t)(nodes->M > 0 ? nodes->M : 0), tu = ths->c2r ? 1 : 2;
  FloatBuf &fh = ths->dev->b[0];
  if (ths->f_hat) {
    if (!upload(fh, ths->f_hat, 2 * (size_t)ths->nfh, s)) return -1;
  } else if (!ensure(fh, 2 * (size_t)ths->nfh) ||
             !cuda_ok(cudaMemsetAsync(fh.d64, 0, sizeof(double) * 2 * (size_t)ths->nfh, s), "memset")) {
    return -1;
  }
  const unsigned flag[3] = {PNFFT_COMPUTE_F, PNFFT_COMPUTE_GRAD_F, PNFFT_COMPUTE_HESSIAN_F};
  float *user[3] = {nodes->f, nodes->grad, nodes->hess};
  const size_t comps[3] = {1, 3, 6};
  double *dptr[3] = {nullptr, nullptr, nullptr};
  const bool acc = (cflags & PNFFT_COMPUTE_ACCUMULATED) != 0;
  for (int k = 0; k < 3; k++) {
    if (!(cflags & flag[k]) || !user[k]) continue;
    FloatBuf &b = nodes->dev->b[1 + k];
    const size_t n = comps[k] * M * tu;
    if (!(acc ? upload(b, user[k], n, s) : ensure(b, n))) return -1;
    dptr[k] = b.d64;
  }
  pnfft_gb300_set_device_arrays(nodes->nd, nodes->dev->b[0].d64, dptr[0], dptr[1], dptr[2]);
  pnfft_gb300_set_device_f_hat(ths->p, fh.d64);
  if (engine_trafo(ths->p, nodes->nd, cflags)) return -1;
  for (int k = 0; k < 3; k++)
    if (dptr[k] && !download(nodes->dev->b[1 + k], user[k], comps[k] * M * tu, s)) return -1;
  return finish(ths) ? 0 : -1;
}

int pnfftf_gb300_adj_dev(pnfftf_plan ths, pnfftf_nodes nodes, unsigned cflags) {
  cudaStream_t s;
  if (!begin(ths, nodes, &s)) return -1;
  const size_t M = (size_t)(nodes->M > 0 ? nodes->M : 0), tu = ths->c2r ? 1 : 2;
  const size_t nf = 2 * (size_t)ths->nfh;
  FloatBuf &fh = ths->dev->b[0];
  if ((cflags & PNFFT_COMPUTE_ACCUMULATED) && ths->f_hat) {
    if (!upload(fh, ths->f_hat, nf, s)) return -1;
  } else if (!ensure(fh, nf)) {
    return -1;
  }
  double *df = nullptr, *dg = nullptr;
  if ((cflags & PNFFT_COMPUTE_F) && nodes->f) {
    if (!upload(nodes->dev->b[1], nodes->f, M * tu, s)) return -1;
    df = nodes->dev->b[1].d64;
  }
  if ((cflags & PNFFT_COMPUTE_GRAD_F) && nodes->grad) {
    if (!upload(nodes->dev->b[2], nodes->grad, 3 * M * tu, s)) return -1;
    dg = nodes->dev->b[2].d64;
  }
  pnfft_gb300_set_device_arrays(nodes->nd, nodes->dev->b[0].d64, df, dg, nullptr);
  pnfft_gb300_set_device_f_hat(ths->p, fh.d64);
  if (engine_adj(ths->p, nodes->nd, cflags)) return -1;
  if (ths->f_hat && !download(fh, ths->f_hat, nf, s)) return -1;
  return finish(ths) ? 0 : -1;
}
