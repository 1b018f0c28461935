// socgpu_internal.h -- device-side tables and launch parameters shared by the
// kernels and the C-ABI layer of libsocgpu.
#pragma once

#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>

#include "../../include/socgpu.h"

namespace socgpu {

// Most absorbers one k-term product may combine (random overlap).
constexpr int kMaxAbsPerBand = 8;
// Planck polynomial degree limit (block 6).
constexpr int kMaxPlanckCoeff = 12;
// Cloud parameters per Pade set (opt_prop_pade_2_mod.F90: 16 coefficients).
constexpr int kPadeParm = 16;
constexpr int kMaxCloudComp = 4;

// One absorber of a band (block 4/5 entries for (band, species)).
struct BandGas {
  int species;     // 0-based species index into gas_mix_ratio
  int i_scale_k;   // ip_scale_band / term / null
  int i_scale_fnc; // ip_scale_power_law / quad / doppler_quad / fnc_null
  int l_doppler;
  double p_ref, t_ref, doppler_cor;
  double scale[4]; // band scaling parameters (ip_scale_band)
  float p_ref_f, t_ref_f, doppler_cor_f, scale_f[4];   // FP32 copies for the mixed kernels
};

struct BandInfo {
  int n_abs;                  // absorbers of the band (0 if l_gas false)
  int g_first, g_count;       // range of g-points (k-term products) of the band
  double solar_flux_band;     // fraction of the solar constant
  double rayleigh_coeff;      // m2/kg
  double planck[kMaxPlanckCoeff];
  float rayleigh_f, solar_flux_band_f;
  float planck_f[kMaxPlanckCoeff];
  BandGas gas[kMaxAbsPerBand];
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
};

// Device-resident spectrum.
struct SpectrumDev {
  int n_band, n_gpoint, n_species, n_deg_fit;
  int nd_band, nd_k_term;           // leading extents of McICA subcol_k tables
  double t_ref_planck;
  int has_solar, has_planck, has_rayleigh;
  int n_drop_type, n_ice_type;
  BandInfo *bands;                  // [n_band]
  GPoint *gpoints;                  // [n_gpoint]
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
  int l_rescale, n_order_forward, l_ir_source_quad, l_rayleigh, l_gas, l_aerosol_mode;
  int l_flux_div, first_band, last_band;
  int mcica;
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
  const double *p, *t, *t_level, *mass, *gas_mix_ratio;
  int nd_species;
  // bound
  const double *zen_0, *solar_irrad, *rho_alb, *t_ground;
  // aerosol
  int n_mode, nd_mode;
  const double *mode_mix_ratio, *mode_absorption, *mode_scattering, *mode_asymmetry;
  // cloud (McICA)
  int n_condensed, n_cloud_type;
  int comp_type[kMaxCloudComp];      // cloud type of each component (1-based)
  int comp_phase[kMaxCloudComp];     // ip_phase_water / ice
  int comp_parm_index[kMaxCloudComp];// 0-based drop or ice type
  const double *condensed_mix_ratio, *condensed_dim_char, *w_cloud, *frac_cloud;
  const double *c_sub, *frac_cloudy;
  const int *n_subcol_cld;
  const int *subcol_k, *first_subcol_k, *subcol_reorder;
  int n_subcol_gen, n_subcol_req, nd_band_sp;
  // outputs
  double *flux_up, *flux_down, *flux_direct, *flux_div, *heating_rate;
  int *error_flag;                  // device flag: set when a bound is violated
};

// Launch configuration chosen by the tuner.
struct TileConfig {
  int lanes_per_solve;   // P: lanes sharing one (column, g-point) solve
  int warps_per_cta;     // warps per CTA; one CTA per column
};

// Kernel entry points (defined in the .cu translation units).
#define SOCGPU_DECL_LAUNCH(name) \
  int name(const FluxParams &p, const TileConfig &cfg, cudaStream_t s, char *msg, size_t len);
SOCGPU_DECL_LAUNCH(launch_flux_fp64_lwns)
SOCGPU_DECL_LAUNCH(launch_flux_fp64_full)
SOCGPU_DECL_LAUNCH(launch_flux_fp64_mcica)
SOCGPU_DECL_LAUNCH(launch_flux_mixed_lwns)
SOCGPU_DECL_LAUNCH(launch_flux_mixed_full)
SOCGPU_DECL_LAUNCH(launch_flux_mixed_mcica)
#undef SOCGPU_DECL_LAUNCH

void count_launch();

}  // namespace socgpu
