// spread_line_f32.cu -- the FP32-mixed instances of the line-wise spreading.
#include "spread_line.cuh"

namespace pg {
bool launch_spread_line_f32(const ConvArgs &a, int mode, cudaStream_t s) { return spread_line_t<float>(a, mode, s); }
}  // namespace pg
