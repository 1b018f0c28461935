// flux_launch.cuh -- dispatch of the templated flux kernel over the tile
// shapes (lanes per solve P, layers per lane CH) it is instantiated for.
#pragma once

#include <cstdio>
#include "flux_kernel.cuh"

namespace socgpu {

template <int P_, int CH_>
struct Shape { static constexpr int P = P_, CH = CH_; };

template <class R, bool MIX, bool NOSCAT, bool MCICA, class S>
int try_launch(const FluxParams &p, const TileConfig &cfg, cudaStream_t st, char *msg, size_t len,
               bool &done) {
  if (done || cfg.lanes_per_solve != S::P || S::P * S::CH < p.n_layer) return 0;
  // the smallest chunk of this P that covers the column is chosen by the
  // caller's ordering of shapes (ascending CH)
  done = true;
  const int nb = p.last_band - p.first_band + 1;
  int max_smem = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // widest band batch (then most warps) whose staging fits in shared memory
  int warps = cfg.warps_per_cta, batch = nb;
  SmemLayout lay{};
  for (;;) {
    lay = make_layout<R>(S::P * S::CH, S::P, batch, p.max_abs, MCICA ? p.n_condensed : 0,
                         MCICA ? p.n_subcol_gen : 0, warps * 32 / S::P, p.isolir == SOCGPU_IP_INFRA_RED, MCICA);
    if ((long long)lay.bytes <= max_smem) break;
    if (batch > 1) { --batch; continue; }
    if (warps > 1) { warps /= 2; batch = nb; continue; }
    snprintf(msg, len, "one band of %d layers needs %zu bytes of shared memory (limit %d)", p.n_layer, lay.bytes,
             max_smem);
    return SOCGPU_I_ERR_RANGE;
  }
  const int threads = warps * 32;
  FluxParams q = p;
  q.band_batch = batch;
  auto kern = flux_kernel<R, MIX, S::P, S::CH, NOSCAT, MCICA>;
  if (lay.bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      snprintf(msg, len, "shared memory request of %zu bytes refused: %s", lay.bytes, cudaGetErrorString(e));
      return SOCGPU_I_ERR_RANGE;
    }
  }
  if (p.n_profile <= 0) return 0;
  kern<<<p.n_profile, threads, lay.bytes, st>>>(q);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, len, "flux kernel launch failed: %s", cudaGetErrorString(e));
    return SOCGPU_I_ABORT_CALCULATION;
  }
  return 0;
}

template <class R, bool MIX, bool NOSCAT, bool MCICA, class... Shapes>
int launch_shapes(const FluxParams &p, const TileConfig &cfg, cudaStream_t st, char *msg, size_t len) {
  bool done = false;
  int status = 0;
  ((status = status ? status : try_launch<R, MIX, NOSCAT, MCICA, Shapes>(p, cfg, st, msg, len, done)), ...);
  if (!done && status == 0) {
    snprintf(msg, len, "no kernel instantiated for %d lanes per solve and %d layers", cfg.lanes_per_solve,
             p.n_layer);
    return SOCGPU_I_ERR_RANGE;
  }
  return status;
}


}  // namespace socgpu

// Shape lists: ascending CH within each P so the first fit is the tightest.
#define SOCGPU_SHAPES_FP64 \
  Shape<16, 4>, Shape<16, 8>, Shape<16, 16>, Shape<32, 4>, Shape<32, 8>, Shape<32, 16>
#define SOCGPU_SHAPES_MIXED                                                                      \
  Shape<8, 8>, Shape<8, 13>, Shape<8, 18>, Shape<16, 4>, Shape<16, 8>, Shape<16, 16>, Shape<32, 4>, \
      Shape<32, 8>, Shape<32, 16>
