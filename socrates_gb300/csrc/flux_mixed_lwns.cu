// Instantiation of the flux kernel: precision mixed, mode lwns.
#include "flux_launch.cuh"

namespace socgpu {
int launch_flux_mixed_lwns(const FluxParams &p, const TileConfig &cfg, cudaStream_t s, char *msg, size_t len) {
  return launch_shapes<float, true, true, false, SOCGPU_SHAPES_MIXED>(p, cfg, s, msg, len);
}
}  // namespace socgpu
