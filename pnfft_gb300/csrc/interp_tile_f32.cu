// interp_tile_f32.cu -- the FP32-mixed instances of the one-warp-per-node interpolation.
#include "interp_tile.cuh"

namespace pg {
bool launch_interp_tile_f32(const ConvArgs &a, int mode, cudaStream_t s) { return interp_tile_t<float>(a, mode, s); }
}  // namespace pg
