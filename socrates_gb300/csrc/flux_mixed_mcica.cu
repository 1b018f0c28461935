// Instantiation of the flux kernel: precision mixed, mode mcica.
#include "flux_launch.cuh"

namespace socgpu {
int launch_flux_mixed_mcica(const FluxParams &p, const TileConfig &cfg, cudaStream_t s, char *msg, size_t len) {
  return launch_shapes<float, true, false, true, SOCGPU_SHAPES_MIXED>(p, cfg, s, msg, len);
}
}  // namespace socgpu
