// spread_line_f64.cu -- the FP64 instances of the line-wise spreading.
#include "spread_line.cuh"

namespace pg {
bool launch_spread_line_f64(const ConvArgs &a, int mode, cudaStream_t s) { return spread_line_t<double>(a, mode, s); }
}  // namespace pg
