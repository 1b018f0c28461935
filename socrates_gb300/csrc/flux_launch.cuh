// flux_launch.cuh -- dispatch of the templated flux kernel over the tile
// shapes (lanes per solve P, layers per lane CH) it is instantiated for.
#pragma once

#include <algorithm>
#include <cstdio>
#include "flux_kernel.cuh"

namespace socgpu {

template <int P_, int CH_>
struct Shape { static constexpr int P = P_, CH = CH_; };

template <class R, bool MIX, bool NOSCAT, bool MCICA, int SRC, class S>
int try_launch(const FluxParams &p, const TileConfig &cfg, cudaStream_t st, char *msg, size_t len,
               bool &done) {
  if (done || cfg.lanes_per_solve != S::P || S::P * S::CH < p.n_layer) return 0;
  if (cfg.chunk && cfg.chunk != S::CH) return 0;
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
    lay = make_layout<R>(p, S::P * S::CH, S::P, batch, warps * 32 / S::P, MCICA,
                         FluxKernel<R, MIX, S::P, S::CH, NOSCAT, MCICA, SRC>::kRawFetch);
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
  auto kern = flux_kernel<R, MIX, S::P, S::CH, NOSCAT, MCICA, SRC>;
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

// Prepare one kernel class of a multi-batch launch for shape S: the band
// batch of every item so that all fit one shared-memory size, the kernel
// attribute, and a persistent grid of the resident CTAs of every SM.
template <class R, bool MIX, bool NOSCAT, bool MCICA, int SRC, class S>
int try_prepare(BatchGroup &g, char *msg, size_t len, bool &done) {
  if (done || g.tile.lanes_per_solve != S::P || g.tile.chunk != S::CH) return 0;
  done = true;
  int max_smem = 0, dev = 0, n_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const int warps = g.tile.warps_per_cta;
  const int n_groups = warps * 32 / S::P;
  auto bytes_of = [&](const FluxParams &p, int batch) {
    return make_layout<R>(p, S::P * S::CH, S::P, batch, n_groups, MCICA,
                          FluxKernel<R, MIX, S::P, S::CH, NOSCAT, MCICA, SRC>::kRawFetch).bytes;
  };
  auto kern = flux_kernel_batched<R, MIX, S::P, S::CH, NOSCAT, MCICA, SRC>;
  // the kernel's static shared memory (its parameter copy) counts against
  // the same per-CTA limit
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) {
    cudaGetLastError();
    snprintf(msg, len, "attributes of the batched kernel not available");
    return SOCGPU_I_ABORT_CALCULATION;
  }
  const size_t dyn_cap = (size_t)max_smem > fa.sharedSizeBytes ? (size_t)max_smem - fa.sharedSizeBytes : 0;
  // the launch's shared memory: the largest whole-spectrum staging of any
  // item, capped at the device limit; items that need more stage their bands
  // in batches
  size_t smem = 0;
  for (int i = 0; i < g.n_items; ++i) {
    const FluxParams &p = g.items[i];
    if (p.n_layer > S::P * S::CH) {
      snprintf(msg, len, "batch %d has %d layers, more than the %d of its tile", i, p.n_layer, S::P * S::CH);
      return SOCGPU_I_ERR_RANGE;
    }
    smem = std::max(smem, bytes_of(p, p.last_band - p.first_band + 1));
  }
  smem = std::min(smem, dyn_cap);
  for (int i = 0; i < g.n_items; ++i) {
    FluxParams &p = g.items[i];
    int batch = p.last_band - p.first_band + 1;
    while (batch > 1 && bytes_of(p, batch) > smem) --batch;
    if (bytes_of(p, batch) > smem) {
      snprintf(msg, len, "batch %d: one band needs %zu bytes of shared memory (limit %zu)", i, bytes_of(p, 1), smem);
      return SOCGPU_I_ERR_RANGE;
    }
    p.band_batch = batch;
  }
  const size_t dyn = smem;
  if (dyn > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) {
      cudaGetLastError();
      snprintf(msg, len, "shared memory request of %zu bytes refused: %s", dyn, cudaGetErrorString(e));
      return SOCGPU_I_ERR_RANGE;
    }
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, dyn);
  if (e != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    snprintf(msg, len, "no CTA of %d threads and %zu bytes fits an SM", warps * 32, dyn);
    return SOCGPU_I_ERR_RANGE;
  }
  g.kernel = (const void *)kern;
  g.smem = dyn;
  g.threads = warps * 32;
  g.grid = (int)std::min<long long>(g.total, (long long)per_sm * n_sm);
  return 0;
}

template <class R, bool MIX, bool NOSCAT, bool MCICA, int SRC, class... Shapes>
int prepare_shapes(BatchGroup &g, char *msg, size_t len) {
  bool done = false;
  int status = 0;
  ((status = status ? status : try_prepare<R, MIX, NOSCAT, MCICA, SRC, Shapes>(g, msg, len, done)), ...);
  if (!done && status == 0) {
    snprintf(msg, len, "no kernel instantiated for %d lanes per solve and %d layers per lane",
             g.tile.lanes_per_solve, g.tile.chunk);
    return SOCGPU_I_ERR_RANGE;
  }
  return status;
}

template <class R, bool MIX, bool NOSCAT, bool MCICA, int SRC, class... Shapes>
int launch_shapes(const FluxParams &p, const TileConfig &cfg, cudaStream_t st, char *msg, size_t len) {
  bool done = false;
  int status = 0;
  ((status = status ? status : try_launch<R, MIX, NOSCAT, MCICA, SRC, Shapes>(p, cfg, st, msg, len, done)), ...);
  if (!done && status == 0) {
    snprintf(msg, len, "no kernel instantiated for %d lanes per solve and %d layers", cfg.lanes_per_solve,
             p.n_layer);
    return SOCGPU_I_ERR_RANGE;
  }
  return status;
}


// The kernels of one source (SOCGPU_IP_SOLAR or SOCGPU_IP_INFRA_RED) over the
// chunk list; the build compiles the two sources as separate objects and the
// infra-red object's entry points hand solar work to the solar one.
template <class R, bool MIX, bool NOSCAT, bool MCICA, int SRC, int P, int... CH>
int launch_chunks(const FluxParams &p, const TileConfig &cfg, cudaStream_t st, char *msg, size_t len) {
  return launch_shapes<R, MIX, NOSCAT, MCICA, SRC, Shape<P, CH>...>(p, cfg, st, msg, len);
}

template <class R, bool MIX, bool NOSCAT, bool MCICA, int SRC, int P, int... CH>
int prepare_chunks(BatchGroup &g, char *msg, size_t len) {
  for (int i = 0; i < g.n_items; ++i)
    if (g.items[i].isolir != SRC) {
      snprintf(msg, len, "a kernel class mixes solar and infra-red batches");
      return SOCGPU_I_ERR_FATAL;
    }
  return prepare_shapes<R, MIX, NOSCAT, MCICA, SRC, Shape<P, CH>...>(g, msg, len);
}

// Load every kernel of the chunk list onto the device now (cudaFuncGetAttributes
// loads a lazily-loaded function): a first launch that loads its module can
// wait for kernels already running, which a request server must not do.
template <class R, bool MIX, bool NOSCAT, bool MCICA, int SRC, int P, int... CH>
int preload_chunks() {
  cudaFuncAttributes a{};
  bool ok = true;
  ((ok = ok && cudaFuncGetAttributes(&a, flux_kernel<R, MIX, P, CH, NOSCAT, MCICA, SRC>) == cudaSuccess), ...);
  ((ok = ok && cudaFuncGetAttributes(&a, flux_kernel_batched<R, MIX, P, CH, NOSCAT, MCICA, SRC>) == cudaSuccess),
   ...);
  if (!ok) cudaGetLastError();
  return ok ? 0 : SOCGPU_I_ABORT_CALCULATION;
}

}  // namespace socgpu
