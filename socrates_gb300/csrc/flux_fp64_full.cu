// Instantiation of the flux kernel: precision fp64, mode full.
#include "flux_launch.cuh"

namespace socgpu {
int launch_flux_fp64_full(const FluxParams &p, const TileConfig &cfg, cudaStream_t s, char *msg, size_t len) {
  return launch_shapes<double, false, false, false, SOCGPU_SHAPES_FP64>(p, cfg, s, msg, len);
}
}  // namespace socgpu
