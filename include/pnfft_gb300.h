/*
 * pnfft_gb300.h -- extensions of libpnfft_gb300 beyond the reference interface.
 *
 * These entry points have no counterpart in the reference (mpip/pnfft); they
 * expose what a GPU implementation adds: error reporting, the arithmetic
 * precision of the device path, device-resident (zero-copy) arrays and
 * streams, and the bit-exact node sort for verification.
 * Included by pnfft.h; may also be included alone.
 */
#ifndef PNFFT_GB300_H
#define PNFFT_GB300_H 1

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef PNFFT_H
typedef struct pnfft_plan_s *pnfft_plan;
typedef struct pnfft_nodes_s *pnfft_nodes;
#endif

/* Precision of the device path of a plan.
 *  PNFFT_GB300_FP64        all of D, F and B in FP64 (default).
 *  PNFFT_GB300_FP32_MIXED  window values, spreading, interpolation and the FFT
 *                          in FP32 with FP32 accumulation; node-to-grid index
 *                          computation, the window Fourier coefficients of D
 *                          and the host-facing arrays stay FP64.
 * PNFFT_GB300_FP32 is a plan flag (a bit unused by the reference's flags)
 * selecting the mixed form at pnfft_init_*. */
#define PNFFT_GB300_FP64 0
#define PNFFT_GB300_FP32_MIXED 1
#define PNFFT_GB300_FP32 (1U << 30)

/* Message of the last error recorded by any call (thread-local), or "" if none;
 * pnfft_gb300_clear_error() resets it.  Errors never fall back to the CPU. */
const char *pnfft_gb300_last_error(void);
void pnfft_gb300_clear_error(void);

/* Number of CUDA devices visible (0 when the driver has none). */
int pnfft_gb300_device_count(void);

/* Select / query the precision of a plan (returns 0 on success). */
int pnfft_gb300_set_precision(pnfft_plan ths, int precision);
int pnfft_gb300_get_precision(const pnfft_plan ths);

/* Run the plan's work on a caller-owned cudaStream_t (NULL = the plan's own
 * stream).  Returns 0 on success.
 * CUDA graphs: pnfft_trafo / pnfft_adj may be captured on that stream once
 * one call with the same plan, node count and flags has run, if the nodes
 * and f_hat are device arrays (below); stage timers are skipped while the
 * stream is capturing.  Host arrays are refused during capture. */
int pnfft_gb300_set_stream(pnfft_plan ths, void *cuda_stream);

/* Convolution kernels of a plan, chosen per plan (e.g. by timing them):
 *  0 = default: B^T along lines of tiles; the FP32-mixed B of f alone along
 *      the same lines, other B one warp per node over a tile (cutoff and
 *      grid permitting);
 *  1 = one thread per node (small node counts on large grids);
 *  2 = the FP32-mixed B one warp per node over 8x8x8 tiles (any output), and
 *      the FP32-mixed B^T of f with the register window that moves by copies;
 *  3 = the FP32-mixed B of f in groups of nodes with overlapping stencils
 *      per warp (the same bits as 2). */
int pnfft_gb300_set_conv_method(pnfft_plan ths, int method);
int pnfft_gb300_get_conv_method(const pnfft_plan ths);
/* The kernel family of the plan's last interpolation B (adjoint = 0) or
 * spreading B^T (adjoint = 1): 0 none yet (or no nodes), 1 groups of nodes
 * per warp (FP32-mixed B), 2 one warp per node over a tile, 3 lines of tiles,
 * 4 one thread per node.  Set when the launch is issued. */
int pnfft_gb300_get_conv_kernel(const pnfft_plan ths, int adjoint);

/* Per-plan autotuning (no counterpart in the reference).  Times, on the
 * given nodes and with the plan's current arrays (host or device), the
 * kernel families of the interpolation (pnfft_trafo with trafo_flags) and of
 * the spreading (pnfft_adj with adj_flags; 0 skips a direction) and the
 * number of nodes per CTA of line binnings (256, 512, 2048), each binning
 * included in its call's time, and keeps the fastest for this plan.  The
 * transforms run as usual (the arrays receive their outputs); a node set
 * whose distribution differs much from later ones may tune differently.
 * pnfft_gb300_get_tuning returns (interpolation method, spreading method,
 * nodes per line sub-problem).  Returns 0 on success. */
int pnfft_gb300_autotune(pnfft_plan ths, pnfft_nodes nodes, unsigned trafo_flags, unsigned adj_flags, int reps);
int pnfft_gb300_get_tuning(const pnfft_plan ths, int *tuning3);
/* Sets the three values of pnfft_gb300_get_tuning (methods 0..3 as in
 * pnfft_gb300_set_conv_method; nodes per line sub-problem a multiple of 32
 * in [32, 4096]), e.g. a tuning saved from an earlier run. */
int pnfft_gb300_set_tuning(pnfft_plan ths, const int *tuning3);

/* Batched convolutions (no counterpart in the reference).  Between
 * pnfft_gb300_batch_begin(stream) and pnfft_gb300_batch_end(), every
 * pnfft_trafo / pnfft_adj (on any stream) with device
 * arrays attached, fixed nodes, an FP32-mixed plan, COMPUTE_F alone, the
 * line kernels (conv method 0; no ik, interlacing, gradient or Hessian) and
 * fewer line sub-problems than 4 CTAs per SM (a call too small to fill the
 * GPU alone; larger calls keep their grid in L2 from D to B) runs
 * its binning and D + F (trafo) or binning and grid clearing (adjoint) at
 * once, each into a grid of its own, and defers its convolution.
 * pnfft_gb300_batch_end makes the batch's stream wait for the deferred calls
 * (an event per call) and launches there, per direction and cutoff, one
 * kernel over the sub-problems of all deferred calls, then the adjoints' F^H
 * and D^T, without synchronizing; the deferred outputs are ready in the
 * batch's stream order.  Other calls run as usual.  The calls
 * of a batch must be independent: none may read an array another one writes;
 * their device arrays must stay allocated until pnfft_gb300_batch_end (a plan
 * or node set that is freed first has its deferred calls run at that point).
 * A batch can be captured into a CUDA graph after one uncaptured run of the
 * same calls (which allocates the grids).  One batch is open at a time per
 * process, and the calls come from one host thread.  Returns 0 on success. */
int pnfft_gb300_batch_begin(void *cuda_stream);
int pnfft_gb300_batch_end(void);
/* Of the last closed batch: the calls whose convolution was deferred, and
 * the batched convolution kernels launched for them. */
int pnfft_gb300_batch_stats(int *deferred_calls, int *launches);

/* Zero-copy mode.  When device arrays are attached, pnfft_trafo/pnfft_adj read
 * and write them directly and return without synchronizing the stream; the
 * host pointers of the plan/nodes are not touched.  Layouts are those of the
 * host arrays.  Pass NULL to detach (back to host arrays). */
int pnfft_gb300_set_device_f_hat(pnfft_plan ths, void *d_f_hat);
int pnfft_gb300_set_device_arrays(pnfft_nodes nodes, double *d_x, void *d_f, void *d_grad_f, void *d_hessian_f);

/* Promise that the node coordinates do not change until the next call with
 * fixed=0 (or until pnfft_set_x / pnfft_gb300_set_device_arrays): the binning
 * of the nodes onto grid tiles is then computed once and reused.
 * pnfft_precompute_psi implies the same promise, as in the reference. */
int pnfft_gb300_nodes_set_fixed(pnfft_nodes nodes, int fixed);

/* Wait for all work of the plan's stream (returns 0 on success). */
int pnfft_gb300_synchronize(pnfft_plan ths);

/* Verification entry points (host arrays in and out, run on the GPU):
 *  - the sort of PNFFT_SORT_NODES: pairs[2p] = key of the p-th node in sorted
 *    order, pairs[2p+1] = its original index (stable, bit-exact with the
 *    reference's radix sort, kernel/ndft-parallel.c:2121-2159);
 *  - the lowest grid index floor(n_t x_t) - m of every node (with the
 *    interlacing shift when interlaced != 0), kernel/ndft-parallel.c:2165-2174,
 *    evaluated the way the plan's binning evaluates it (FP64 arithmetic, or the
 *    integer-only form of FP32-mixed plans). */
int pnfft_gb300_sort_nodes(pnfft_plan ths, ptrdiff_t M, const double *x, long long *pairs);
int pnfft_gb300_node_index(pnfft_plan ths, ptrdiff_t M, const double *x, int interlaced, long long *u);

/* The sort of pnfft_gb300_sort_nodes without any device allocation.  It has
 * no counterpart in the reference; it exists for callers that cannot allocate
 * device memory where they sort (a fixed memory pool or arena that must not
 * grow, an allocator that forbids cudaMalloc because of its implicit
 * synchronisation, or memory reserved in full up front).
 *  - d_x (3M doubles) and d_pairs (2M long longs, same layout as
 *    pnfft_gb300_sort_nodes) are device arrays of the current device; only
 *    the plan's n and m are read.
 *  - The scratch is one static device array of this library, sized for at
 *    most PNFFT_GB300_SORT_NOALLOC_MAX_NODES nodes (4.5 MiB); a larger M is
 *    refused with an error (-1).
 *  - The first call on a device resolves the array's address on that device
 *    (the device must be current), and so does the first call after the
 *    device's context was re-created (cudaDeviceReset); make that call before
 *    any stream capture.
 *  - The work is queued on cuda_stream (NULL: the legacy default stream) and
 *    the call returns without synchronizing.
 *  - All calls share the array: calls whose work overlaps on the GPU race and
 *    give wrong results; order them on one stream.
 * Returns 0 on success. */
#define PNFFT_GB300_SORT_NOALLOC_MAX_NODES 262144
int pnfft_gb300_sort_nodes_noalloc(const pnfft_plan ths, ptrdiff_t M, const double *d_x, long long *d_pairs,
                                   void *cuda_stream);

/* The charge/dipole sequence of a particle-mesh code in one call; the
 * reference runs it as four calls in tests/check_charge_dipole.c:151-233:
 *   pnfft_adj(plan, charges, PNFFT_COMPUTE_F);
 *   pnfft_adj(plan, dipoles, PNFFT_COMPUTE_GRAD_F);      (added to f_hat)
 *   pnfft_trafo(plan, charges, PNFFT_COMPUTE_F | PNFFT_COMPUTE_GRAD_F);
 *   pnfft_trafo(plan, dipoles, PNFFT_COMPUTE_GRAD_F | PNFFT_COMPUTE_HESSIAN_F);
 * followed by the per-particle energies and forces.  Inputs: the charges in
 * charges->f at charges->x, the dipole moments in dipoles->grad_f at
 * dipoles->x (host arrays; a c2c plan).  On return the node arrays and the
 * plan's f_hat hold what the four calls leave there, and, where not NULL,
 * energy[Mc + Md] = (q phi, mu . grad phi) and force[3 (Mc + Md)] =
 * (q grad phi, H mu).  Each node set is copied to the GPU and binned once for
 * both of its transforms, and f_hat stays on the GPU between them.
 * compute_flags may add PNFFT_OMIT_* flags.  Returns 0 on success. */
int pnfft_gb300_charge_dipole(pnfft_plan ths, pnfft_nodes charges, pnfft_nodes dipoles, unsigned compute_flags,
                              void *energy, void *force);

/* Measurement aid, no counterpart in the reference: the FP32 multiply-add
 * rate of the current device in TFLOP/s (2 flops per multiply-add), timed with
 * CUDA events over a kernel of independent FMA chains on every SM: scalar
 * FFMA (paired = 0) or the paired FP32 FMA of sm_100+ (paired = 1), the
 * instruction of the spreading and interpolation kernels.  Allocates 4 KiB of
 * device memory for the result sink.  Returns 0 on success. */
int pnfft_gb300_measure_fp32_fma(int paired, double *tflops);

/* Milliseconds of the stages of the last pnfft_trafo / pnfft_adj of the plan,
 * indexed like the PNFFT_TIMER_* constants. */
int pnfft_gb300_last_stage_ms(const pnfft_plan ths, int adjoint, double *ms10);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* PNFFT_GB300_H */
