// flux_phased.cu -- launches of the phased flux kernel (flux_phased.cuh) for
// one precision and one mode, chosen at compile time:
//   -DSOCGPU_PREC=0|1   (FP64 | mixed FP32 with FP64 I/O)
//   -DSOCGPU_MODE=0|1   (infra-red without scattering | full scattering)
// The layer capacity of the staging (64, 128 or 256 slots) is the smallest
// that covers the column.
#include <algorithm>
#include <cstdio>
#include "flux_phased.cuh"

#if !defined(SOCGPU_PREC) || !defined(SOCGPU_MODE)
#error "compile with -DSOCGPU_PREC and -DSOCGPU_MODE"
#endif
#if SOCGPU_PREC == 0
#define SOCGPU_R double
#define SOCGPU_MIX false
#else
#define SOCGPU_R float
#define SOCGPU_MIX true
#endif
#define SOCGPU_PASTE_(a, p, m) a##_##p##_##m
#define SOCGPU_PASTE(a, p, m) SOCGPU_PASTE_(a, p, m)

namespace socgpu {
namespace {

template <class R, bool MIX, bool NOSCAT, int SRC, int LPM>
int launch_phased_lp(const FluxParams &p, const TileConfig &cfg, cudaStream_t st, char *msg, size_t len) {
  using K = PhasedKernel<R, MIX, NOSCAT, SRC, LPM>;
  int max_smem = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int nb = p.last_band - p.first_band + 1;
  // k-terms per batch (the tile's chunk; at most 32, the lanes of the warp
  // that runs the recurrences), then the widest band batch that fits; halve
  // the k-term batch if one band does not fit
  int gb = cfg.chunk > 0 ? std::min(cfg.chunk, 32) : 16;
  int batch = nb;
  size_t bytes = 0;
  for (;;) {
    bytes = make_layout<R>(p, LPM, 1, batch, 1, false).bytes + K::extra_bytes(p.n_layer, gb);
    if ((long long)bytes <= max_smem) break;
    if (batch > 1) { --batch; continue; }
    if (gb > 1) { gb /= 2; batch = nb; continue; }
    snprintf(msg, len, "one band of %d layers needs %zu bytes of shared memory (limit %d)", p.n_layer, bytes,
             max_smem);
    return SOCGPU_I_ERR_RANGE;
  }
  FluxParams q = p;
  q.band_batch = batch;
  auto kern = flux_kernel_phased<R, MIX, NOSCAT, SRC, LPM>;
  if (bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      snprintf(msg, len, "shared memory request of %zu bytes refused: %s", bytes, cudaGetErrorString(e));
      return SOCGPU_I_ERR_RANGE;
    }
  }
  if (p.n_profile <= 0) return 0;
  // warp 0 runs the serial recurrences, the others the coefficients and sums
  const int warps = cfg.warps_per_cta > 0 ? std::max(2, std::min(cfg.warps_per_cta, 8)) : 8;
  kern<<<p.n_profile, warps * 32, bytes, st>>>(q, gb);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, len, "phased flux kernel launch failed: %s", cudaGetErrorString(e));
    return SOCGPU_I_ABORT_CALCULATION;
  }
  return 0;
}

template <class R, bool MIX, bool NOSCAT, int SRC>
int launch_phased_src(const FluxParams &p, const TileConfig &cfg, cudaStream_t st, char *msg, size_t len) {
  if (p.n_layer <= 64) return launch_phased_lp<R, MIX, NOSCAT, SRC, 64>(p, cfg, st, msg, len);
  if (p.n_layer <= 128) return launch_phased_lp<R, MIX, NOSCAT, SRC, 128>(p, cfg, st, msg, len);
  if (p.n_layer <= kPhasedMaxLayers) return launch_phased_lp<R, MIX, NOSCAT, SRC, 256>(p, cfg, st, msg, len);
  snprintf(msg, len, "the phased kernel covers at most %d layers (%d given)", kPhasedMaxLayers, p.n_layer);
  return SOCGPU_I_ERR_RANGE;
}

}  // namespace

int SOCGPU_PASTE(launch_phased, SOCGPU_PREC, SOCGPU_MODE)(const FluxParams &p, const TileConfig &cfg,
                                                          cudaStream_t s, char *msg, size_t len) {
#if SOCGPU_MODE == 0
  return launch_phased_src<SOCGPU_R, SOCGPU_MIX, true, SOCGPU_IP_INFRA_RED>(p, cfg, s, msg, len);
#else
  if (p.isolir == SOCGPU_IP_INFRA_RED)
    return launch_phased_src<SOCGPU_R, SOCGPU_MIX, false, SOCGPU_IP_INFRA_RED>(p, cfg, s, msg, len);
  return launch_phased_src<SOCGPU_R, SOCGPU_MIX, false, SOCGPU_IP_SOLAR>(p, cfg, s, msg, len);
#endif
}

}  // namespace socgpu
