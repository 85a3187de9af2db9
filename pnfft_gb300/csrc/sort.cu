// sort.cu -- node keys and the stable node sort of PNFFT_SORT_NODES, and the
// node-to-grid index, on the device.
//
// Reference: sort_nodes_for_better_cache_handle (kernel/ndft-parallel.c:
// 2121-2159): key = ((u0 n1 + u1) n2 + u2) with u_t = floor(n_t x_t - m) mod
// n_t, sorted by the stable LSD radix sort of util/util.c:200-275 (9-bit
// digits over bits [0, ceil(log2(n0 n1 n2)) - 1]).  The device sort below runs
// the same digit passes; each pass is a stable counting sort (per-block digit
// histograms, a digit-major scan over blocks, and an in-order scatter in which
// a warp ranks equal digits with __match_any_sync), so the permutation is
// identical to the reference's.
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

#include "pg_index.cuh"
#include "pg_internal.h"
#include "pg_kernels.h"

namespace pg {

__global__ void k_node_index(const double *__restrict__ x, int64_t M, int n0, int n1, int n2, int m, int il,
                             long long *__restrict__ u) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const int n[3] = {n0, n1, n2};
  for (int t = 0; t < 3; t++) {
    double xs = x[3 * j + t];
    if (il) xs = __dadd_rn(xs, __ddiv_rn(0.5, (double)n[t]));
    double fnx = floor(__dmul_rn((double)n[t], xs));
    u[3 * j + t] = (long long)fnx - m;
  }
}

// the integer-only evaluation used by the FP32-mixed binning
__global__ void k_node_index_exact(const double *__restrict__ x, int64_t M, int n0, int n1, int n2, int m,
                                   long long *__restrict__ u) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const int n[3] = {n0, n1, n2};
  for (int t = 0; t < 3; t++) {
    long long fnx;
    float fr;
    nx_exact(x[3 * j + t], n[t], &fnx, &fr);
    u[3 * j + t] = fnx - m;
  }
}

void launch_node_index(const double *x, int64_t M, const int *n, int m, int il, bool integer_path, long long *u,
                       cudaStream_t s) {
  if (M <= 0) return;
  if (integer_path && !il) k_node_index_exact<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(x, M, n[0], n[1], n[2], m, u);
  else k_node_index<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(x, M, n[0], n[1], n[2], m, il, u);
}

// key of ndft-parallel.c:2131-2142; n*x - m evaluated without FMA
__global__ void k_sort_keys(const double *__restrict__ x, int64_t M, int n0, int n1, int n2, int m,
                            long long *__restrict__ pairs) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  const int n[3] = {n0, n1, n2};
  long long key = 0;
  for (int j = 0; j < 3; j++) {
    long long h = (long long)floor(__dsub_rn(__dmul_rn((double)n[j], x[3 * i + j]), (double)m));
    long long uj = (h % n[j] + n[j]) % n[j];
    key += uj;
    if (j + 1 < 3) key *= n[j + 1];
  }
  pairs[2 * i] = key;
  pairs[2 * i + 1] = i;
}

constexpr int kDigits = 512;
constexpr int kBlockItems = 1024;  // items per block (one warp walks them in order)

__global__ void k_radix_hist(const long long *__restrict__ in, int64_t M, int shift, int nblocks,
                             int *__restrict__ hist) {
  __shared__ int h[kDigits];
  for (int d = threadIdx.x; d < kDigits; d += blockDim.x) h[d] = 0;
  __syncthreads();
  int64_t lo = (int64_t)blockIdx.x * kBlockItems;
  int64_t hi = min((int64_t)M, lo + kBlockItems);
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) atomicAdd(&h[(in[2 * i] >> shift) & (kDigits - 1)], 1);
  __syncthreads();
  for (int d = threadIdx.x; d < kDigits; d += blockDim.x) hist[(int64_t)d * nblocks + blockIdx.x] = h[d];
}

// exclusive scan of hist (digit-major), single CTA
__global__ void __launch_bounds__(1024) k_radix_scan(int *hist, int64_t total) {
  __shared__ long long part[1024];
  const int tid = threadIdx.x;
  const int64_t chunk = (total + 1023) / 1024;
  const int64_t lo = min(total, (int64_t)tid * chunk), hi = min(total, lo + chunk);
  long long s = 0;
  for (int64_t i = lo; i < hi; i++) s += hist[i];
  part[tid] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    long long v = (tid >= off) ? part[tid - off] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  long long p = part[tid] - s;
  for (int64_t i = lo; i < hi; i++) {
    int c = hist[i];
    hist[i] = (int)p;
    p += c;
  }
}

// one warp per block scatters its items in order; equal digits within a
// 32-item chunk are ranked by lane order
__global__ void k_radix_scatter(const long long *__restrict__ in, long long *__restrict__ out, int64_t M, int shift,
                                int nblocks, const int *__restrict__ offs) {
  __shared__ int run[kDigits];
  const int lane = threadIdx.x;
  for (int d = lane; d < kDigits; d += 32) run[d] = offs[(int64_t)d * nblocks + blockIdx.x];
  __syncwarp();
  int64_t lo = (int64_t)blockIdx.x * kBlockItems;
  int64_t hi = min((int64_t)M, lo + kBlockItems);
  for (int64_t c = lo; c < hi; c += 32) {
    int64_t i = c + lane;
    bool valid = i < hi;
    long long key = valid ? in[2 * i] : 0;
    long long idx = valid ? in[2 * i + 1] : 0;
    int d = valid ? (int)((key >> shift) & (kDigits - 1)) : -1 - lane;
    unsigned act = __ballot_sync(0xffffffffu, valid);
    unsigned peers = __match_any_sync(0xffffffffu, d) & act;
    int rank = __popc(peers & ((1u << lane) - 1));
    int basepos = 0;
    if (valid) basepos = run[d];
    __syncwarp();
    if (valid) {
      int pos = basepos + rank;
      out[2 * (int64_t)pos] = key;
      out[2 * (int64_t)pos + 1] = idx;
      // the highest-ranked lane of each digit advances the running offset
      if ((peers >> lane) == 1u) run[d] = basepos + rank + 1;
    }
    __syncwarp();
  }
}

int radix_sort_nodes(const double *x, int64_t M, const int *n, int m, long long *pairs_dev, cudaStream_t s) {
  if (M <= 0) return 0;
  k_sort_keys<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(x, M, n[0], n[1], n[2], m, pairs_dev);
  double nprod = (double)n[0] * (double)n[1] * (double)n[2];
  long long rhigh = (long long)ceil(log2(nprod)) - 1;
  int nblocks = (int)((M + kBlockItems - 1) / kBlockItems);
  long long *tmp = nullptr;
  int *hist = nullptr;
  if (cudaMallocAsync(&tmp, sizeof(long long) * 2 * M, s) != cudaSuccess) return -1;
  if (cudaMallocAsync(&hist, sizeof(int) * (size_t)kDigits * nblocks, s) != cudaSuccess) {
    cudaFreeAsync(tmp, s);
    return -1;
  }
  long long *from = pairs_dev, *to = tmp;
  int shift = 0;
  while (rhigh >= 0) {
    k_radix_hist<<<nblocks, 256, 0, s>>>(from, M, shift, nblocks, hist);
    k_radix_scan<<<1, 1024, 0, s>>>(hist, (int64_t)kDigits * nblocks);
    k_radix_scatter<<<nblocks, 32, 0, s>>>(from, to, M, shift, nblocks, hist);
    long long *t = from;
    from = to;
    to = t;
    shift += 9;
    rhigh -= 9;
  }
  if (from != pairs_dev) cudaMemcpyAsync(pairs_dev, from, sizeof(long long) * 2 * M, cudaMemcpyDeviceToDevice, s);
  cudaFreeAsync(tmp, s);
  cudaFreeAsync(hist, s);
  return 0;
}

// ---------------------------------------------------------------------------
// The node sort without any device allocation.
//
// Some callers cannot allocate device memory at the point where they sort:
// code running under a device memory pool or arena that it must not grow, an
// allocator hook that forbids cudaMalloc/cudaMallocAsync (their implicit
// synchronisation or pool growth would stall a latency-bound loop), or a
// process whose device memory is fully reserved up front.  For them the sort
// below takes its scratch -- the ping-pong copy of the (key, index) pairs and
// the per-block digit histograms -- from one statically sized device array
// instead of cudaMallocAsync.  The array is part of this module's device
// image and exists once per device; its address is resolved with
// cudaGetSymbolAddress by the first call made in each CUDA context (with that
// context's device current): once per device, and once more after the
// context has been destroyed and re-created (cudaDeviceReset), since a new
// context loads the module at another address.  That first call may load the
// module, so make it before any stream capture in the context.  The array
// holds at most kNoAllocMaxNodes nodes; larger calls are refused with an
// error and must use the allocating sort.
//
// Every call shares the array and finds the previous call's contents in it.
// Nothing there has to start at zero: every radix pass writes each digit
// count of every block (k_radix_hist) and each of the M pairs (the stable
// scatter is a permutation) before reading them.  Calls whose work overlaps
// on the GPU (different streams, or threads on the same device without
// ordering) race on the array and give wrong results; order them on one
// stream or synchronize between them.
// ---------------------------------------------------------------------------
constexpr int64_t kNoAllocMaxNodes = int64_t(1) << 18;
constexpr int kNoAllocMaxBlocks = (int)(kNoAllocMaxNodes / kBlockItems);
constexpr size_t kNoAllocPairBytes = sizeof(long long) * 2 * (size_t)kNoAllocMaxNodes;  // 4 MiB
constexpr size_t kNoAllocHistBytes = sizeof(int) * (size_t)kDigits * kNoAllocMaxBlocks;  // 512 KiB
static __device__ __align__(256) unsigned char g_sort_scratch[kNoAllocPairBytes + kNoAllocHistBytes];

static_assert(kNoAllocPairBytes % 256 == 0, "histograms start 256-byte aligned");

constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_scratch_mu;
// per device: the scratch address and the unique ID of the context it was resolved in
static void *g_scratch_ptr[kNoAllocMaxDevices] = {};
static unsigned long long g_scratch_ctx[kNoAllocMaxDevices] = {};

// the unique ID of the current context (cuCtxGetId, CUDA 12.0+, reached
// through the runtime's driver entry points so that no libcuda link is needed)
static int current_context_id(unsigned long long *id) {
  typedef CUresult (*get_current_t)(CUcontext *);
  typedef CUresult (*get_id_t)(CUcontext, unsigned long long *);
  static get_current_t get_current = nullptr;
  static get_id_t get_id = nullptr;
  if (!get_current || !get_id) {
    void *f0 = nullptr, *f1 = nullptr;
    cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
      return -1;
    get_current = (get_current_t)f0;
    get_id = (get_id_t)f1;
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, id) != CUDA_SUCCESS) return -1;
  return 0;
}

static int sort_scratch_address(void **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaSetDevice(dev);  // initialises the primary context and makes it current
  if (e != cudaSuccess) {
    set_error("pnfft_gb300_sort_nodes_noalloc: no usable CUDA device: %s", cudaGetErrorString(e));
    return -1;
  }
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    set_error("pnfft_gb300_sort_nodes_noalloc: device %d is beyond the %d devices supported", dev, kNoAllocMaxDevices);
    return -1;
  }
  unsigned long long ctx = 0;
  if (current_context_id(&ctx)) {
    set_error("pnfft_gb300_sort_nodes_noalloc: the current CUDA context of device %d could not be identified", dev);
    return -1;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_sort_scratch);
    if (e != cudaSuccess || !ptr) {
      set_error("pnfft_gb300_sort_nodes_noalloc: cudaGetSymbolAddress of the scratch array failed on device %d: %s",
                dev, cudaGetErrorString(e));
      return -1;
    }
    g_scratch_ptr[dev] = ptr;
    g_scratch_ctx[dev] = ctx;
  }
  *out = g_scratch_ptr[dev];
  return 0;
}

}  // namespace pg

extern "C" int pnfft_gb300_sort_nodes_noalloc(const pnfft_plan ths, ptrdiff_t M, const double *d_x, long long *d_pairs,
                                              void *cuda_stream) {
  using namespace pg;
  if (!ths) {
    set_error("pnfft_gb300_sort_nodes_noalloc: plan is NULL");
    return -1;
  }
  if (M < 0 || M > kNoAllocMaxNodes) {
    set_error("pnfft_gb300_sort_nodes_noalloc: M=%td is outside [0, %lld], the capacity of the static scratch; "
              "use pnfft_gb300_sort_nodes for larger node sets",
              M, (long long)kNoAllocMaxNodes);
    return -1;
  }
  if (M == 0) return 0;
  if (!d_x || !d_pairs) {
    set_error("pnfft_gb300_sort_nodes_noalloc: d_x and d_pairs must be device arrays");
    return -1;
  }
  void *scratch = nullptr;
  if (sort_scratch_address(&scratch)) return -1;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  long long *tmp = (long long *)scratch;
  int *hist = (int *)((unsigned char *)scratch + kNoAllocPairBytes);
  const int n0 = (int)ths->n[0], n1 = (int)ths->n[1], n2 = (int)ths->n[2];
  k_sort_keys<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(d_x, M, n0, n1, n2, ths->m, d_pairs);
  const double nprod = (double)n0 * (double)n1 * (double)n2;
  long long rhigh = (long long)ceil(log2(nprod)) - 1;
  const int nblocks = (int)((M + kBlockItems - 1) / kBlockItems);
  long long *from = d_pairs, *to = tmp;
  int shift = 0;
  while (rhigh >= 0) {
    k_radix_hist<<<nblocks, 256, 0, s>>>(from, M, shift, nblocks, hist);
    k_radix_scan<<<1, 1024, 0, s>>>(hist, (int64_t)kDigits * nblocks);
    k_radix_scatter<<<nblocks, 32, 0, s>>>(from, to, M, shift, nblocks, hist);
    long long *t = from;
    from = to;
    to = t;
    shift += 9;
    rhigh -= 9;
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && from != d_pairs)
    e = cudaMemcpyAsync(d_pairs, from, sizeof(long long) * 2 * M, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) {
    set_error("pnfft_gb300_sort_nodes_noalloc: launch failed: %s", cudaGetErrorString(e));
    return -1;
  }
  return 0;
}
