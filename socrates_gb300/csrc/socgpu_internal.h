// socgpu_internal.h -- device-side tables and launch parameters shared by the
// kernels and the C-ABI layer of libsocgpu.
#pragma once

#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>

#include "../../include/socgpu.h"

namespace socgpu {

// Most absorbers one k-term product may combine (random overlap).
constexpr int kMaxAbsPerBand = 12;
// Planck polynomial degree limit (block 6).
constexpr int kMaxPlanckCoeff = 12;
// Coefficients kept per cloud parameter set: the most any supported scheme
// reads (Pade: 16, opt_prop_pade_2_mod.F90; Fu: 14; Slingo-Schrecker: 6).
constexpr int kCloudParm = 16;
constexpr int kMaxCloudComp = 4;

// Self-broadened absorbers whose gas fractions a column stages (lookup tables).
constexpr int kMaxSb = 4;

// Classic aerosol: mixing-ratio entries a launch takes (radiatively active
// ones), and the widest humidity table and phase-function moments per entry.
constexpr int kMaxAerMr = 32;
// Most gas species a flux kernel fetches ahead of staging (more: direct loads).
constexpr int kMaxRawGas = 8;

// One absorber of a band (block 4/5 entries for (band, species)).
struct BandGas {
  int species;     // 0-based species index into gas_mix_ratio
  int i_scale_k;   // ip_scale_band / term / null
  int i_scale_fnc; // ip_scale_power_law / quad / doppler_quad / wenyi / lookup / t_lookup / fnc_null
  int l_doppler;
  int sb;          // lookup tables: 0-based self-broadened index (staged gas fraction), -1 none
  int n_t;         // temperature-only tables: entries of the species' temperature grid
  double p_ref, t_ref, doppler_cor;
  double scale[4]; // band scaling parameters (ip_scale_band)
  float p_ref_f, t_ref_f, doppler_cor_f, scale_f[4];   // FP32 copies for the mixed kernels
};

// One continuum of a band (blocks 8 and 9; rescale_continuum.F90).
constexpr int kMaxContPerBand = 4;
struct BandCont {
  int type;                   // SOCGPU_IP_SELF_CONTINUUM / SOCGPU_IP_FRN_CONTINUUM
  int fnc;                    // ip_scale_power_law / ip_scale_power_quad
  double p_ref, t_ref, k, scale[3];
  float p_ref_f, t_ref_f, k_f, scale_f[3];
};

struct BandInfo {
  int n_abs;                  // absorbers of the band (0 if l_gas false)
  int n_cont;                 // continua of the band
  BandCont cont[kMaxContPerBand];
  int g_first, g_count;       // range of g-points (k-term products) of the band
  double solar_flux_band;     // fraction of the solar constant
  double rayleigh_coeff;      // m2/kg
  double planck[kMaxPlanckCoeff];
  float rayleigh_f, solar_flux_band_f;
  float planck_f[kMaxPlanckCoeff];
  BandGas gas[kMaxAbsPerBand];
  // equivalent extinction (k_eqv_scl): the k-terms of absorber j >= 1 are
  // TermK entries minor_first[j] .. minor_first[j] + minor_count[j] - 1
  int minor_first[kMaxAbsPerBand], minor_count[kMaxAbsPerBand];
};

// One k-term of one absorber of a band: the minor gases of k_eqv_scl.
struct TermK {
  int iex;                          // 0-based k-term
  int lk_off;                       // offset of its lookup table in k_lookup, -1 without
  double k, w;
  double scale[4];                  // per-term scaling parameters (ip_scale_term)
  float kf, wf, scale_f[4];
};

// One g-point: a k-term product of random overlap
// (solve_band_random_overlap.F90:533-560).
struct GPoint {
  int band;                         // 0-based
  int iex_major;                    // 0-based k-term of the first absorber
  int n_abs;
  float pad;
  double weight;                    // product weight of the term
  double k[kMaxAbsPerBand];         // k of each absorber's term
  double term_scale[kMaxAbsPerBand][4];   // per-term scaling parameters (ip_scale_term)
  float weight_f;                   // FP32 copies for the mixed kernels
  float kf[kMaxAbsPerBand];
  float term_scale_f[kMaxAbsPerBand][4];
  int lk_off[kMaxAbsPerBand];       // offset of each absorber's lookup table in k_lookup, -1 without
  short iex[kMaxAbsPerBand];        // each absorber's 0-based k-term (Wen-Yi tables)
};

// Device-resident spectrum.
struct SpectrumDev {
  int n_band, n_gpoint, n_species, n_deg_fit;
  int nd_band, nd_k_term;           // leading extents of McICA subcol_k tables
  double t_ref_planck;
  int has_solar, has_planck, has_rayleigh, has_continuum, index_water;
  int n_drop_type, n_ice_type;
  BandInfo *bands;                  // [n_band]
  GPoint *gpoints;                  // [n_gpoint]
  int random_ok;                    // the random-overlap products fit SOCGPU_MAX_GPOINT
  // equivalent extinction: the major absorber's terms as g-points, the minor
  // absorbers' terms as TermK entries
  BandInfo *bands_keqv;
  GPoint *gpoints_keqv;
  TermK *minor_terms;
  int n_gpoint_keqv;
  int host_first_g_keqv[SOCGPU_MAX_BAND + 1];
  // lookup tables: P/T grid, gas fractions, compact k tables, temperature-only grids
  int has_lookup, lk_n_pre, lk_n_tmp, lk_n_gf, n_sb;
  double *lk_grid;                  // ln p [n_pre], T [n_pre][n_tmp], gas fractions [n_gf]
  float *lk_grid_f;
  double *k_lookup;
  float *k_lookup_f;
  int sb_species[kMaxSb];           // 0-based species of each self-broadened index
  double sb_ratio_gas[kMaxSb], ratio_water;
  int l_water;
  int nd_t_lookup_gas;
  double *t_lookup_gas;             // [n_species][nd_t_lookup_gas]
  float *t_lookup_gas_f;
  // Wen-Yi tables packed as plg[26], ttb[10], tto[9], gk250b[n4], gk4[10][26][n4], gk6[9][26][n6]
  int wenyi_n4, wenyi_n6;
  double *wenyi;
  float *wenyi_f;
  // classic aerosol species (block 11): per band, species and humidity the
  // row (absorption, scattering, phase-function moments 1..aer_nphf)
  int aer_n_species, aer_nh, aer_nphf;
  double *aer_tab;                  // [n_band][aer_n_species][aer_nh][2 + aer_nphf]
  float *aer_tab_f;
  double *aer_hum;                  // [aer_n_species][aer_nh] humidities of each species' rows
  float *aer_hum_f;
  double *drop_parm;                // [n_drop_type][n_band][16]
  double *ice_parm;                 // [n_ice_type][n_band][16]
  float *drop_parm_f, *ice_parm_f;  // FP32 copies
  // host copies for validation
  int host_first_g[SOCGPU_MAX_BAND + 1];
};

// Everything a flux kernel launch reads, as device pointers with the
// caller's Fortran leading extents.
struct FluxParams {
  // control
  int isolir, i_2stream, i_scatter_method, i_direct_tau;
  float scheme_f[5];                 // the mixed kernels' constants of i_2stream (SchemeF: A, B, C, D, K)
  int l_rescale, n_order_forward, l_ir_source_quad, l_rayleigh, l_gas, l_aerosol_mode;
  int l_flux_div, first_band, last_band;
  int mcica;                         // cloud fields staged (McICA or cloud regions)
  int region;                        // clear and cloudy regions (ip_cloud_mix_max / mix_random)
  int solver_hogan;                  // regions solved by solver_mix_direct_hogan, else solver_mix_direct
  int l_continuum, l_mixing_ratio, i_water;   // i_water: 0-based species of water vapour
  // sizes
  int n_profile, n_layer, nd_profile, nd_layer, id_ct;  // id_ct 0-based first cloudy layer
  int g_begin, g_end;               // g-point range of the band range
  int max_abs;                      // most absorbers of any band in the range (>= 1)
  int band_batch;                   // bands staged in shared memory at a time (set by the launcher)
  // spectrum
  const BandInfo *bands;
  const GPoint *gpoints;
  const double *drop_parm, *ice_parm;
  const float *drop_parm_f, *ice_parm_f;
  int n_band, n_deg_fit;
  double t_ref_planck;
  float t_ref_planck_f;
  const double *weight_band;        // device copy, [n_band]
  // atm
  const double *p, *t, *t_level, *mass, *gas_mix_ratio, *density;
  int nd_species;
  // bound
  const double *zen_0, *solar_irrad, *rho_alb, *t_ground;
  const double *flux_ground;        // (nd_profile, nd_band) surface Planck flux per band, or null
  // aerosol
  int n_mode, nd_mode;
  const double *mode_mix_ratio, *mode_absorption, *mode_scattering, *mode_asymmetry;
  // cloud (McICA)
  int n_condensed, n_cloud_type;
  int comp_type[kMaxCloudComp];      // cloud type of each component (1-based)
  int comp_phase[kMaxCloudComp];     // ip_phase_water / ice
  int comp_parm_index[kMaxCloudComp];// 0-based drop or ice type
  int comp_scheme[kMaxCloudComp];    // parametrization (ip_slingo_schrecker, ip_drop_pade_2, ...)
  const double *condensed_mix_ratio, *condensed_dim_char, *w_cloud, *frac_cloud;
  const double *c_sub, *frac_cloudy;
  const int *n_subcol_cld;
  const int *subcol_k, *first_subcol_k, *subcol_reorder;
  int n_subcol_gen, n_subcol_req, nd_band_sp;
  // classic aerosol (opt_prop_aerosol.F90): the active mixing-ratio entries
  int l_aerosol, n_aer_mr, l_hg;    // l_hg: Henyey-Greenstein moments for every species
  int aer_n_species, aer_nh, aer_nphf, aer_nh_common;
  int aer_entry[kMaxAerMr];         // third index of aer_mix_ratio of each active entry
  int aer_species[kMaxAerMr];       // its 0-based species
  int aer_parm[kMaxAerMr];          // the species' SOCGPU_IP_AEROSOL_PARAM_*
  double aer_dhum;                  // humidity step of the common table, 1 / (aer_nh_common - 1)
  float aer_dhum_f;
  const double *aer_mix_ratio;      // (nd_profile, nd_layer, nd_aerosol_mr)
  const double *mean_rel_humidity;  // (nd_profile, nd_layer), moist species only
  const double *aer_tab, *aer_hum;
  const float *aer_tab_f, *aer_hum_f;
  // prescribed aerosol optical properties (prsc_opt_prop.F90) of the
  // unparametrized species of the active entries: the data on their levels,
  // and the per-layer sums the prescribed-property kernel writes before the
  // flux kernel runs
  int l_aer_prsc, n_prsc, prsc_nq;  // prsc_nq: phase-function moments interpolated
  int nd_prof_prsc, nd_lev_prsc, nd_phf_prsc, nd_sp_prsc;
  int prsc_species[kMaxAerMr];      // 0-based species
  int prsc_count[kMaxAerMr];        // active entries that name it
  int prsc_nlev[kMaxAerMr];         // its levels
  const double *prsc_p, *prsc_abs, *prsc_scat, *prsc_phf;
  // [n_profile][4][last_band - first_band + 1][n_layer]: absorption,
  // scattering, scattering x asymmetry, scattering x forward moment
  const double *aer_prsc;
  // outputs
  double *flux_up, *flux_down, *flux_direct, *flux_div, *heating_rate;
  int *error_flag;                  // device flag: set when a bound is violated
  // equivalent extinction (k_eqv_scl): minor absorbers folded into grey absorption
  int keqv, l_grey_single;
  int term_scr;                     // a scratch row per group: per-term scaled absorbers or k_eqv
  const TermK *minor_terms;
  // lookup-table k scaling: the column stages interpolation factors
  int lk_on, lk_n_pre, lk_n_tmp, lk_n_gf, n_sb;
  const double *lk_grid, *k_lookup;
  const float *lk_grid_f, *k_lookup_f;
  int sb_species[kMaxSb];
  double sb_ratio_gas[kMaxSb], ratio_water;
  int l_water;
  int nd_t_lookup_gas;
  const double *t_lookup_gas;
  const float *t_lookup_gas_f;
  int wenyi_n4, wenyi_n6;
  const double *wenyi;
  const float *wenyi_f;
  // cloud regions: overlap of like regions and the three-region types
  int corr_mode;                     // like regions at an interface: 0 random, 1 maximal, 2 exp(dp / dp_corr)
  double dp_corr[3];                 // decorrelation scales [Pa] of the clear, stratiform, convective regions
  int triple;                        // three regions: clear, stratiform and convective (ip_cloud_triple)
  int type_region[4];                // the region (2 stratiform, 3 convective) of each 0-based cloud type
};

// Launch configuration chosen by the tuner.
struct TileConfig {
  int lanes_per_solve;   // P: lanes sharing one (column, g-point) solve
  int warps_per_cta;     // warps per CTA; one CTA per column
  int chunk;             // CH: layers per lane; 0 = the smallest instantiated chunk that covers the column
};

// One kernel class of a multi-batch launch: the batches that share precision,
// mode and tile, run by one persistent launch of flux_kernel_batched.
struct BatchGroup {
  int precision = 0, mode = 0;
  TileConfig tile{};
  FluxParams *items = nullptr;        // host array [n_items] (band_batch filled by the prepare step)
  long long *col_start = nullptr;     // host array [n_items + 1]
  int n_items = 0;
  long long total = 0;                // columns of all batches
  // filled by the prepare step
  const void *kernel = nullptr;
  size_t smem = 0;
  int threads = 0, grid = 0;
};

// Layers per lane (CH) instantiated for each precision and lane count P; a
// kernel covers P * CH layers.  flux_inst.cu is compiled once per
// (precision, mode, P) and instantiates these chunks.
#define SOCGPU_CHUNKS_MIXED_8  5, 8, 13, 18
#define SOCGPU_CHUNKS_MIXED_16 3, 4, 5, 7, 9, 16
#define SOCGPU_CHUNKS_MIXED_32 3, 4, 5, 8, 16
#define SOCGPU_CHUNKS_FP64_16  4, 8, 16
#define SOCGPU_CHUNKS_FP64_32  4, 5, 8, 16

// The chunks of (precision, lanes) in ascending order; returns their count
// (0 when that lane count is not built for the precision).
inline int chunk_list(int precision, int lanes, const int **out) {
  static const int m8[] = {SOCGPU_CHUNKS_MIXED_8}, m16[] = {SOCGPU_CHUNKS_MIXED_16},
                   m32[] = {SOCGPU_CHUNKS_MIXED_32}, d16[] = {SOCGPU_CHUNKS_FP64_16},
                   d32[] = {SOCGPU_CHUNKS_FP64_32};
#define SOCGPU_RET(a) do { *out = a; return (int)(sizeof(a) / sizeof(a[0])); } while (0)
  if (precision == SOCGPU_PRECISION_MIXED) {
    if (lanes == 8) SOCGPU_RET(m8);
    if (lanes == 16) SOCGPU_RET(m16);
    if (lanes == 32) SOCGPU_RET(m32);
  } else {
    if (lanes == 16) SOCGPU_RET(d16);
    if (lanes == 32) SOCGPU_RET(d32);
  }
#undef SOCGPU_RET
  *out = nullptr;
  return 0;
}

// Smallest built chunk of (precision, lanes) covering n_layer, or 0.
inline int smallest_chunk(int precision, int lanes, int n_layer) {
  const int *c = nullptr;
  const int n = chunk_list(precision, lanes, &c);
  for (int i = 0; i < n; ++i)
    if (lanes * c[i] >= n_layer) return c[i];
  return 0;
}

// Kernel entry points, one pair per (precision 0 fp64 / 1 mixed, mode
// 0 lwns / 1 full / 2 mcica, lanes), defined by the objects of flux_inst.cu.
#define SOCGPU_DECL_FLUX(prec, mode, lanes)                                                             \
  int launch_flux_##prec##_##mode##_##lanes(const FluxParams &p, const TileConfig &cfg, cudaStream_t s, \
                                            char *msg, size_t len);                                    \
  int prepare_flux_##prec##_##mode##_##lanes(BatchGroup &g, char *msg, size_t len);                     \
  int preload_flux_##prec##_##mode##_##lanes();
#define SOCGPU_DECL_FLUX_MODES(prec, lanes) \
  SOCGPU_DECL_FLUX(prec, 0, lanes) SOCGPU_DECL_FLUX(prec, 1, lanes) SOCGPU_DECL_FLUX(prec, 2, lanes)
SOCGPU_DECL_FLUX_MODES(0, 16)
SOCGPU_DECL_FLUX_MODES(0, 32)
SOCGPU_DECL_FLUX_MODES(1, 8)
SOCGPU_DECL_FLUX_MODES(1, 16)
SOCGPU_DECL_FLUX_MODES(1, 32)
#undef SOCGPU_DECL_FLUX_MODES
#undef SOCGPU_DECL_FLUX

// The phased kernel (flux_phased.cu), one launcher per (precision, mode
// 0 lwns / 1 full); its tile is lanes_per_solve = 1, chunk = k-terms per batch.
#define SOCGPU_DECL_PHASED(prec, mode)                                                                  \
  int launch_phased_##prec##_##mode(const FluxParams &p, const TileConfig &cfg, cudaStream_t s, char *msg, \
                                    size_t len);
SOCGPU_DECL_PHASED(0, 0)
SOCGPU_DECL_PHASED(0, 1)
SOCGPU_DECL_PHASED(1, 0)
SOCGPU_DECL_PHASED(1, 1)
#undef SOCGPU_DECL_PHASED

// The prescribed-aerosol kernel (aerosol_prsc.cu): bytes of its output for
// a launch, and its launch into `out` on stream st.
size_t prsc_bytes(const FluxParams &p);
int launch_prsc(const FluxParams &p, double *out, cudaStream_t st, char *msg, size_t len);

// Whether the phased kernel covers a launch: clear sky, no equivalent
// extinction, the direct beam delta-scaled, at most 256 layers.
constexpr int kPhasedMaxLayers = 256;
inline bool phased_supported(const FluxParams &p) {
  return !p.mcica && !p.keqv && p.n_layer <= kPhasedMaxLayers &&
         !(p.isolir == SOCGPU_IP_SOLAR && p.i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING);
}

void count_launch();

}  // namespace socgpu
