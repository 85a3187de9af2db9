// api_float.h -- the objects of the single-precision API pnfftf_*
// (api_float.cpp) and its device side (float_io.cu).
#pragma once
#include <stddef.h>

#include "../../include/pnfft.h"

namespace pg {
struct FloatDev;  // float_io.cu: device buffers and stream of a float plan / nodes
void float_dev_free(FloatDev *d);
}  // namespace pg

struct pnfftf_plan_s {
  pnfft_plan p;     // double plan (its host f_hat is not used by the transforms)
  float *f_hat;     // caller's or own interleaved complex float array
  int own_f_hat;
  ptrdiff_t nfh;    // complex entries of f_hat (local_N total)
  int c2r;
  pg::FloatDev *dev;  // stream and device f_hat (float and double)
};

struct pnfftf_nodes_s {
  pnfft_nodes nd;   // double nodes; the transforms attach device arrays to them
  ptrdiff_t M;
  float *x, *f, *grad, *hess;  // caller's or own float arrays (complex: interleaved)
  pg::FloatDev *dev;  // device x, f, grad, hess (float and double)
};

// float_io.cu: pnfftf_trafo / pnfftf_adj on the GPU; 0 or -1 (error set)
int pnfftf_gb300_trafo_dev(pnfftf_plan ths, pnfftf_nodes nodes, unsigned compute_flags);
int pnfftf_gb300_adj_dev(pnfftf_plan ths, pnfftf_nodes nodes, unsigned compute_flags);
