// interp_tile_f64.cu -- the FP64 instances of the one-warp-per-node interpolation.
#include "interp_tile.cuh"

namespace pg {
bool launch_interp_tile_f64(const ConvArgs &a, int mode, cudaStream_t s) { return interp_tile_t<double>(a, mode, s); }
}  // namespace pg
