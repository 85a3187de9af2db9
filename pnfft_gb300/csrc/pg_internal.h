// pg_internal.h -- host-side plan and node objects of libpnfft_gb300.
//
// Mirrors the reference's plan_s / nodes_s (kernel/ipnfft.h:160-256) for a
// 1x1x1 mesh: what the reference keeps in FP64 host memory (sizes, window
// shape b, interpolation tables, the deconvolution factors) stays on the host
// here as well and is uploaded once; the per-call arrays live on the GPU.
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/pnfft.h"

namespace pg {
struct DevState;    // engine.cu
struct NodeDev;     // engine.cu
}  // namespace pg

struct pnfft_plan_s {
  int d;
  int64_t N[3], n[3], no[3];
  int m, cutoff;
  double x_max[3], sigma[3], b[3];
  unsigned pnfft_flags, pfft_flags;
  int c2r;
  int64_t local_N[3], local_N_start[3], local_N_total;
  int64_t local_no[3], local_no_start[3];
  void *f_hat;      // host array (user's or PNFFT_MALLOC_F_HAT)
  int own_f_hat;
  int window;       // pg::WindowKind
  int gauss_t;      // PNFFT_WINDOW_GAUSSIAN_T
  int intpol_order; // -1: direct evaluation
  int64_t intpol_K;
  std::vector<double> tab[3][3];  // [derivative][axis] interpolation tables
  std::vector<double> inv[3];     // inv_phi_hat per axis over the stored block
  double timer_trafo[PNFFT_TIMER_LENGTH];
  double timer_adj[PNFFT_TIMER_LENGTH];
  double last_ms[2][PNFFT_TIMER_LENGTH];
  int precision;      // PNFFT_GB300_FP64 / PNFFT_GB300_FP32_MIXED
  int conv_method[2];  // [interpolation, spreading]: pnfft_gb300_set_conv_method (both),
                       // or per direction by pnfft_gb300_autotune
  int line_sub_max;    // nodes of a line per CTA (sub-problem) in line binnings
  int last_conv[2];   // pg::ConvKernel of the last B / B^T launch
  void *d_f_hat_user; // zero-copy f_hat
  void *user_stream;
  uint64_t uid;
  uint64_t table_version;  // bumps when b or precision change
  pg::DevState *dev;
};

struct pnfft_nodes_s {
  int64_t local_M;
  double *x, *f, *grad_f, *hessian_f;  // host arrays (complex interleaved for c2c)
  unsigned precompute_flags;
  int fixed;          // coordinates promised constant (binning reused)
  uint64_t version;   // bumps whenever the coordinates may have changed
  uint64_t uid;
  // zero-copy device arrays
  double *u_x;
  void *u_f, *u_grad, *u_hess;
  pg::NodeDev *dev;
};

namespace pg {

// errors (api.cpp)
void set_error(const char *fmt, ...);
const char *last_error();

// engine.cu
int engine_trafo(pnfft_plan ths, pnfft_nodes nodes, unsigned cflags);
int engine_adj(pnfft_plan ths, pnfft_nodes nodes, unsigned cflags);
int engine_autotune(pnfft_plan ths, pnfft_nodes nodes, unsigned trafo_flags, unsigned adj_flags, int reps);
int engine_charge_dipole(pnfft_plan ths, pnfft_nodes charges, pnfft_nodes dipoles, unsigned cflags, void *energy,
                         void *force);
int engine_set_stream(pnfft_plan ths, void *stream);
int engine_batch_begin(void *stream);
int engine_batch_end();
void engine_batch_stats(int *deferred, int *launches);
int engine_sync(pnfft_plan ths);
void engine_release_plan(pnfft_plan ths);
void engine_release_nodes(pnfft_nodes nodes);
int engine_sort_nodes(pnfft_plan ths, int64_t M, const double *x, long long *pairs);
int engine_node_index(pnfft_plan ths, int64_t M, const double *x, int interlaced, long long *u);
int engine_device_count();
void *engine_host_alloc(size_t bytes);
bool engine_host_free(void *p);
void engine_flush_timers(pnfft_plan ths);

}  // namespace pg
