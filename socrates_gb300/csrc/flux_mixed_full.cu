// Instantiation of the flux kernel: precision mixed, mode full.
#include "flux_launch.cuh"

namespace socgpu {
int launch_flux_mixed_full(const FluxParams &p, const TileConfig &cfg, cudaStream_t s, char *msg, size_t len) {
  return launch_shapes<float, true, false, false, SOCGPU_SHAPES_MIXED>(p, cfg, s, msg, len);
}
}  // namespace socgpu
