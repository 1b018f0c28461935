// flux_inst.cu -- instantiation of the flux kernels for one precision, one
// mode and one lane count, chosen at compile time:
//   -DSOCGPU_PREC=0|1   (FP64 | mixed FP32 with FP64 I/O)
//   -DSOCGPU_MODE=0|1|2 (infra-red without scattering | full | McICA)
//   -DSOCGPU_LANES=8|16|32
// The build compiles this file once per combination, in parallel; each
// object defines launch_flux_<prec>_<mode>_<lanes> (one batch, one CTA per
// column) and prepare_flux_<prec>_<mode>_<lanes> (a class of a multi-batch
// launch) over the chunks listed for that precision and lane count.
#include "flux_launch.cuh"

#if !defined(SOCGPU_PREC) || !defined(SOCGPU_MODE) || !defined(SOCGPU_LANES)
#error "compile with -DSOCGPU_PREC, -DSOCGPU_MODE and -DSOCGPU_LANES"
#endif

#if SOCGPU_PREC == 0
#define SOCGPU_R double
#define SOCGPU_MIX false
#if SOCGPU_LANES == 16
#define SOCGPU_CHUNKS SOCGPU_CHUNKS_FP64_16
#elif SOCGPU_LANES == 32
#define SOCGPU_CHUNKS SOCGPU_CHUNKS_FP64_32
#else
#error "FP64 kernels are built for 16 and 32 lanes"
#endif
#else
#define SOCGPU_R float
#define SOCGPU_MIX true
#if SOCGPU_LANES == 8
#define SOCGPU_CHUNKS SOCGPU_CHUNKS_MIXED_8
#elif SOCGPU_LANES == 16
#define SOCGPU_CHUNKS SOCGPU_CHUNKS_MIXED_16
#elif SOCGPU_LANES == 32
#define SOCGPU_CHUNKS SOCGPU_CHUNKS_MIXED_32
#else
#error "mixed kernels are built for 8, 16 and 32 lanes"
#endif
#endif

#define SOCGPU_PASTE_(a, p, m, l) a##_##p##_##m##_##l
#define SOCGPU_PASTE(a, p, m, l) SOCGPU_PASTE_(a, p, m, l)

namespace socgpu {

int SOCGPU_PASTE(launch_flux, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)(const FluxParams &p, const TileConfig &cfg,
                                                                      cudaStream_t s, char *msg, size_t len) {
  return launch_chunks<SOCGPU_R, SOCGPU_MIX, SOCGPU_MODE == 0, SOCGPU_MODE == 2, SOCGPU_LANES, SOCGPU_CHUNKS>(
      p, cfg, s, msg, len);
}

int SOCGPU_PASTE(prepare_flux, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)(BatchGroup &g, char *msg, size_t len) {
  return prepare_chunks<SOCGPU_R, SOCGPU_MIX, SOCGPU_MODE == 0, SOCGPU_MODE == 2, SOCGPU_LANES, SOCGPU_CHUNKS>(
      g, msg, len);
}

}  // namespace socgpu
