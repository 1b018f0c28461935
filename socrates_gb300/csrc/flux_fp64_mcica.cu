// Instantiation of the flux kernel: precision fp64, mode mcica.
#include "flux_launch.cuh"

namespace socgpu {
int launch_flux_fp64_mcica(const FluxParams &p, const TileConfig &cfg, cudaStream_t s, char *msg, size_t len) {
  return launch_shapes<double, false, false, true, SOCGPU_SHAPES_FP64>(p, cfg, s, msg, len);
}
}  // namespace socgpu
