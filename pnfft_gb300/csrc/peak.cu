// peak.cu -- measurement aid: the FP32 multiply-add rate of the device.
//
// The spreading and interpolation kernels are bound by FP32 multiply-adds
// (paired FFMA2 for complex-by-real updates), not by HBM, so their roofline is
// the FP32 FMA rate.  This kernel runs kChains independent multiply-add chains
// per thread on every SM and reports flops per second (2 per multiply-add).
// It has no counterpart in the reference.
#include <cuda_runtime.h>

#include "pg_internal.h"

namespace pg {

constexpr int kChains = 8;
constexpr int kIters = 4096;

template <int PAIRED>
__global__ void __launch_bounds__(256) k_fma_rate(float *sink, float seed) {
  float2 a[kChains];
  const float2 m = make_float2(0.999999f, 1.000001f);
  const float2 c = make_float2(1e-7f, -1e-7f);
#pragma unroll
  for (int k = 0; k < kChains; k++) a[k] = make_float2(seed + k + threadIdx.x, seed - k);
#pragma unroll 1
  for (int it = 0; it < kIters; it++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) {
      if (PAIRED) {
        a[k] = __ffma2_rn(a[k], m, c);
      } else {
        a[k].x = fmaf(a[k].x, m.x, c.x);
        a[k].y = fmaf(a[k].y, m.y, c.y);
      }
    }
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += a[k].x + a[k].y;
  if (s == 12345.678f) sink[threadIdx.x] = s;  // never true; keeps the chains live
}

int measure_fp32_fma(int paired, double *tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                cudaSuccess) {
    set_error("pnfft_gb300_measure_fp32_fma: no CUDA device");
    return -1;
  }
  float *sink = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaMalloc(&sink, 4096) != cudaSuccess || cudaEventCreate(&a) != cudaSuccess ||
      cudaEventCreate(&b) != cudaSuccess) {
    set_error("pnfft_gb300_measure_fp32_fma: device set-up failed");
    cudaFree(sink);
    return -1;
  }
  const int blocks = sms * 8, threads = 256;  // 64 warps per SM
  float best = 1e30f;
  for (int rep = 0; rep < 5; rep++) {
    cudaEventRecord(a, 0);
    if (paired) k_fma_rate<1><<<blocks, threads>>>(sink, 1.0f);
    else k_fma_rate<0><<<blocks, threads>>>(sink, 1.0f);
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (rep > 0 && ms < best) best = ms;  // the first launch is a warm-up
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  if (e != cudaSuccess) {
    set_error("pnfft_gb300_measure_fp32_fma: %s", cudaGetErrorString(e));
    return -1;
  }
  // two FP32 multiply-adds per chain and iteration (re and im), 2 flops each
  const double flops = (double)blocks * threads * kIters * kChains * 2 * 2;
  *tflops = flops / (best * 1e-3) / 1e12;
  return 0;
}

}  // namespace pg

extern "C" int pnfft_gb300_measure_fp32_fma(int paired, double *tflops) {
  if (!tflops) return -1;
  return pg::measure_fp32_fma(paired, tflops);
}
