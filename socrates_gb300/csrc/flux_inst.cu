// flux_inst.cu -- instantiation of the flux kernels for one precision, one
// mode, one lane count and one source, chosen at compile time:
//   -DSOCGPU_PREC=0|1   (FP64 | mixed FP32 with FP64 I/O)
//   -DSOCGPU_MODE=0|1|2 (infra-red without scattering | full | McICA)
//   -DSOCGPU_LANES=8|16|32
//   -DSOCGPU_SRC=1|2    (solar | infra-red; mode 0 is infra-red only)
// The build compiles this file once per combination, in parallel.  The
// infra-red object defines launch_flux_<prec>_<mode>_<lanes> (one batch, one
// CTA per column) and prepare_flux_<prec>_<mode>_<lanes> (a class of a
// multi-batch launch) over the chunks listed for that precision and lane
// count, and passes solar work to the solar object's
// launch_flux_solar_<prec>_<mode>_<lanes> / prepare_flux_solar_...;
// preload_flux_<prec>_<mode>_<lanes> loads all of their kernels.
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

#if !defined(SOCGPU_SRC) || (SOCGPU_SRC != SOCGPU_IP_SOLAR && SOCGPU_SRC != SOCGPU_IP_INFRA_RED) || \
    (SOCGPU_MODE == 0 && SOCGPU_SRC != SOCGPU_IP_INFRA_RED)
#error "compile with -DSOCGPU_SRC=1 (solar, modes 1 and 2) or 2 (infra-red)"
#endif

#define SOCGPU_PASTE_(a, p, m, l) a##_##p##_##m##_##l
#define SOCGPU_PASTE(a, p, m, l) SOCGPU_PASTE_(a, p, m, l)
#define SOCGPU_NOSCAT (SOCGPU_MODE == 0)
#define SOCGPU_MCICA (SOCGPU_MODE == 2)

namespace socgpu {

int SOCGPU_PASTE(launch_flux_solar, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)(const FluxParams &p,
                                                                            const TileConfig &cfg, cudaStream_t s,
                                                                            char *msg, size_t len);
int SOCGPU_PASTE(prepare_flux_solar, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)(BatchGroup &g, char *msg, size_t len);
int SOCGPU_PASTE(preload_flux_solar, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)();

#if SOCGPU_SRC == SOCGPU_IP_SOLAR
int SOCGPU_PASTE(launch_flux_solar, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)(const FluxParams &p,
                                                                            const TileConfig &cfg, cudaStream_t s,
                                                                            char *msg, size_t len) {
  return launch_chunks<SOCGPU_R, SOCGPU_MIX, SOCGPU_NOSCAT, SOCGPU_MCICA, SOCGPU_IP_SOLAR, SOCGPU_LANES,
                       SOCGPU_CHUNKS>(p, cfg, s, msg, len);
}

int SOCGPU_PASTE(prepare_flux_solar, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)(BatchGroup &g, char *msg, size_t len) {
  return prepare_chunks<SOCGPU_R, SOCGPU_MIX, SOCGPU_NOSCAT, SOCGPU_MCICA, SOCGPU_IP_SOLAR, SOCGPU_LANES,
                        SOCGPU_CHUNKS>(g, msg, len);
}

int SOCGPU_PASTE(preload_flux_solar, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)() {
  return preload_chunks<SOCGPU_R, SOCGPU_MIX, SOCGPU_NOSCAT, SOCGPU_MCICA, SOCGPU_IP_SOLAR, SOCGPU_LANES,
                        SOCGPU_CHUNKS>();
}
#else
// The source picks the kernel at run time; the no-scatter family is
// infra-red only.
int SOCGPU_PASTE(launch_flux, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)(const FluxParams &p, const TileConfig &cfg,
                                                                      cudaStream_t s, char *msg, size_t len) {
#if SOCGPU_MODE != 0
  if (p.isolir != SOCGPU_IP_INFRA_RED)
    return SOCGPU_PASTE(launch_flux_solar, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)(p, cfg, s, msg, len);
#endif
  return launch_chunks<SOCGPU_R, SOCGPU_MIX, SOCGPU_NOSCAT, SOCGPU_MCICA, SOCGPU_IP_INFRA_RED, SOCGPU_LANES,
                       SOCGPU_CHUNKS>(p, cfg, s, msg, len);
}

int SOCGPU_PASTE(prepare_flux, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)(BatchGroup &g, char *msg, size_t len) {
#if SOCGPU_MODE != 0
  if (g.n_items > 0 && g.items[0].isolir != SOCGPU_IP_INFRA_RED)
    return SOCGPU_PASTE(prepare_flux_solar, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)(g, msg, len);
#endif
  return prepare_chunks<SOCGPU_R, SOCGPU_MIX, SOCGPU_NOSCAT, SOCGPU_MCICA, SOCGPU_IP_INFRA_RED, SOCGPU_LANES,
                        SOCGPU_CHUNKS>(g, msg, len);
}

int SOCGPU_PASTE(preload_flux, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)() {
  int st = preload_chunks<SOCGPU_R, SOCGPU_MIX, SOCGPU_NOSCAT, SOCGPU_MCICA, SOCGPU_IP_INFRA_RED, SOCGPU_LANES,
                          SOCGPU_CHUNKS>();
#if SOCGPU_MODE != 0
  if (st == 0) st = SOCGPU_PASTE(preload_flux_solar, SOCGPU_PREC, SOCGPU_MODE, SOCGPU_LANES)();
#endif
  return st;
}
#endif

}  // namespace socgpu
