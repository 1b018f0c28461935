"""ctypes mirror of include/socgpu.h.

The same structures bind the product library (libsocgpu.so) and, in the
tests, the CPU oracle, so both receive byte-identical argument blocks.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

# status codes (rad_pcf.F90:391-405)
I_NORMAL, I_ERR_FATAL, I_ABORT_CALCULATION, I_ERR_IO, I_ERR_RANGE, I_ERR_EXIST = 0, 1, 2, 4, 5, 6

# option identifiers (rad_pcf.F90 values)
IP_SOLAR, IP_INFRA_RED = 1, 2
IP_TWO_STREAM = 1
IP_EDDINGTON, IP_DISCRETE_ORD, IP_IFM, IP_PIFM85 = 2, 4, 5, 6
IP_ELSASSER, IP_2S_TEST, IP_HEMI_MEAN, IP_PIFM80 = 12, 14, 15, 16
IP_SCATTER_FULL, IP_NO_SCATTER_ABS, IP_NO_SCATTER_EXT = 1, 2, 3
IP_DIRECT_NOSCALING, IP_DIRECT_DELTA_SCALING, IP_DIRECT_CSR_SCALING = 0, 1, 2
IP_SOLVER_NO_SCAT, IP_SOLVER_HOMOGEN_DIRECT = 2, 13
IP_CLOUD_CLEAR, IP_CLOUD_MCICA = 5, 10
IP_CLOUD_MIX_MAX, IP_CLOUD_MIX_RANDOM = 2, 4
IP_SOLVER_MIX_DIRECT, IP_SOLVER_MIX_DIRECT_HOGAN = 11, 16
IP_CLOUD_TRIPLE, IP_SOLVER_TRIPLE_HOGAN = 6, 17      # three regions: clear, stratiform, convective
IP_CLOUD_PART_CORR, IP_CLOUD_PART_CORR_CNV = 7, 8    # like regions correlated over a pressure scale
IP_CLOUD_TYPE_STRAT, IP_CLOUD_TYPE_CONV = 1, 2
IP_CLOUD_TYPE_SW, IP_CLOUD_TYPE_SI, IP_CLOUD_TYPE_CW, IP_CLOUD_TYPE_CI = 1, 2, 3, 4
IP_CLOUD_HOMOGEN = 1
IP_CLOUD_ICE_WATER = 2
IP_CLOUD_TYPE_WATER, IP_CLOUD_TYPE_ICE = 1, 2
IP_PHASE_WATER, IP_PHASE_ICE = 1, 2
IP_CLCMP_ST_WATER, IP_CLCMP_ST_ICE, IP_CLCMP_CNV_WATER, IP_CLCMP_CNV_ICE = 1, 2, 3, 4
IP_DROP_PADE_2, IP_ICE_PADE_2_PHF = 5, 20
IP_SLINGO_SCHRECKER, IP_SLINGO_SCHRECKER_ICE, IP_ICE_FU_PHF = 1, 1, 12
IP_OVERLAP_HYBRID, IP_OVERLAP_RANDOM = 0, 2
IP_OVERLAP_K_EQV_SCL, IP_OVERLAP_K_EQV, IP_OVERLAP_K_EQV_MOD = 4, 5, 6
IP_SCALE_NULL, IP_SCALE_BAND, IP_SCALE_TERM = 0, 1, 2
IP_SCALE_FNC_NULL, IP_SCALE_POWER_LAW, IP_SCALE_POWER_QUAD, IP_SCALE_DOPPLER_QUAD = 0, 1, 2, 3
IP_SCALE_WENYI, IP_SCALE_LOOKUP, IP_SCALE_T_LOOKUP = 4, 9, 10
IP_RAYLEIGH_TOTAL = 1
IP_AEROSOL_PARAM_DRY, IP_AEROSOL_PARAM_MOIST, IP_AEROSOL_UNPARAMETRIZED = 1, 2, 3
IP_AEROSOL_PARAM_PHF_DRY, IP_AEROSOL_PARAM_PHF_MOIST = 4, 5
IP_AERSRC_CUSACK_RON, IP_AERSRC_CLASSIC_RON, IP_AERSRC_ARCL_RON = 0, 1, 2
IP_MAX_RAND, IP_RAND, IP_EXPONENTIAL, IP_EXPONENTIAL_RAND = 0, 1, 2, 3
IP_MCICA_FULL_SAMPLING, IP_MCICA_SINGLE_SAMPLING, IP_MCICA_OPTIMAL_SAMPLING = 0, 1, 2

PRECISION_FP64, PRECISION_MIXED = 0, 1
RNG_LCG, RNG_PHILOX = 0, 1
NOALLOC_MAX_CLOUD_LAYERS = 1024   # SOCGPU_NOALLOC_MAX_CLOUD_LAYERS
ABI_VERSION = 7
IP_SELF_CONTINUUM, IP_FRN_CONTINUUM = 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class SpectrumDesc(C.Structure):
    _fields_ = [
        ("nd_band", C.c_int), ("nd_species", C.c_int), ("nd_k_term", C.c_int), ("nd_scale_variable", C.c_int),
        ("nd_thermal_coeff", C.c_int), ("nd_drop_type", C.c_int), ("nd_ice_type", C.c_int),
        ("nd_cloud_parameter", C.c_int),
        ("n_band", C.c_int),
        ("wavelength_short", _dp), ("wavelength_long", _dp),
        ("solar_flux_band", _dp), ("i_rayleigh_scheme", C.c_int), ("rayleigh_coeff", _dp),
        ("n_absorb", C.c_int), ("type_absorb", _ip), ("n_band_absorb", _ip), ("index_absorb", _ip),
        ("i_band_k", _ip), ("i_scale_k", _ip), ("i_scale_fnc", _ip),
        ("k", _dp), ("w", _dp), ("scale", _dp), ("p_ref", _dp), ("t_ref", _dp),
        ("l_doppler", _ip), ("doppler_cor", _dp),
        ("n_deg_fit", C.c_int), ("t_ref_planck", C.c_double), ("thermal_coeff", _dp),
        ("l_drop_type", _ip), ("i_drop_parm", _ip), ("drop_parm_list", _dp),
        ("l_ice_type", _ip), ("i_ice_parm", _ip), ("ice_parm_list", _dp),
        ("nd_continuum", C.c_int), ("n_band_continuum", _ip), ("index_continuum", _ip), ("index_water", C.c_int),
        ("i_scale_fnc_cont", _ip), ("k_cont", _dp), ("scale_cont", _dp), ("p_ref_cont", _dp), ("t_ref_cont", _dp),
        # lookup-table k scaling (the '_k' companion file)
        ("n_pre", C.c_int), ("n_tmp", C.c_int), ("p_lookup", _dp), ("t_lookup", _dp), ("k_lookup", _dp),
        ("index_sb", _ip), ("nd_species_sb", C.c_int), ("n_gas_frac", C.c_int), ("gf_lookup", _dp),
        ("k_lookup_sb", _dp), ("molar_weight", _dp),
        ("nd_t_lookup_gas", C.c_int), ("n_t_lookup_gas", _ip), ("t_lookup_gas", _dp), ("k_t_lookup_gas", _dp),
        # CO2/O3 tables of ip_scale_wenyi
        ("wenyi_n_term4", C.c_int), ("wenyi_n_term6", C.c_int), ("wenyi_plg", _dp), ("wenyi_ttb", _dp),
        ("wenyi_tto", _dp), ("wenyi_gk250b", _dp), ("wenyi_gk4", _dp), ("wenyi_gk6", _dp),
        # classic aerosol species (block 11)
        ("n_aerosol", C.c_int), ("nd_aerosol_species", C.c_int), ("nd_humidity", C.c_int),
        ("nd_phase_term", C.c_int), ("type_aerosol", _ip), ("i_aerosol_parm", _ip), ("nhumidity", _ip),
        ("n_aerosol_phf_term", _ip), ("aerosol_humidities", _dp), ("aerosol_abs", _dp), ("aerosol_scat", _dp),
        ("aerosol_phf", _dp),
        ("drop_parm_min_dim", _dp), ("drop_parm_max_dim", _dp), ("ice_parm_min_dim", _dp), ("ice_parm_max_dim", _dp),
        ("i_overlap", _ip),
    ]


class Control(C.Structure):
    _fields_ = [
        ("isolir", C.c_int), ("i_angular_integration", C.c_int), ("i_2stream", C.c_int),
        ("i_scatter_method", C.c_int), ("i_solver", C.c_int), ("i_cloud", C.c_int),
        ("i_cloud_representation", C.c_int), ("i_gas_overlap", C.c_int), ("i_direct_tau", C.c_int),
        ("l_rescale", C.c_int), ("n_order_forward", C.c_int), ("l_ir_source_quad", C.c_int),
        ("l_rayleigh", C.c_int), ("l_gas", C.c_int), ("l_aerosol_mode", C.c_int), ("l_flux_div", C.c_int),
        ("first_band", C.c_int), ("last_band", C.c_int), ("weight_band", _dp), ("precision", C.c_int),
        ("l_continuum", C.c_int), ("l_mixing_ratio", C.c_int), ("l_grey_single", C.c_int),
        ("l_aerosol", C.c_int), ("l_henyey_greenstein_pf", C.c_int),
    ]


class Dimen(C.Structure):
    _fields_ = [
        ("nd_profile", C.c_int), ("nd_layer", C.c_int), ("id_cloud_top", C.c_int), ("nd_aerosol_mode", C.c_int),
        ("nd_cloud_component", C.c_int), ("nd_cloud_type", C.c_int), ("nd_subcol_gen", C.c_int),
        ("nd_subcol_req", C.c_int), ("nd_aerosol_mr", C.c_int),
        ("nd_profile_aerosol_prsc", C.c_int), ("nd_opt_level_aerosol_prsc", C.c_int),
        ("nd_phf_term_aerosol_prsc", C.c_int),
    ]


class Atm(C.Structure):
    _fields_ = [
        ("n_profile", C.c_int), ("n_layer", C.c_int),
        ("p", _dp), ("t", _dp), ("p_level", _dp), ("t_level", _dp), ("mass", _dp), ("gas_mix_ratio", _dp),
        ("density", _dp),
    ]


RUNES_N_GAS = 80
RUNES_N_AER = 33
IP_CLOUD_CONV_STRAT, IP_CLOUD_CSIW, IP_CLOUD_OFF = 3, 4, 5
IP_CLOUD_COMBINE_HOMOGEN, IP_CLOUD_COMBINE_ICE_WATER, IP_CLOUD_SPLIT_HOMOGEN, IP_CLOUD_SPLIT_ICE_WATER = 6, 7, 8, 9
IP_MAX_ENTRAPMENT, IP_ZERO_ENTRAPMENT = 1, 2
IP_HOMOGENEOUS, IP_SCALING, IP_MCICA, IP_TRIPLECLOUDS_2019 = 0, 1, 2, 4
IP_RE_EXTERNAL, IP_RE_LIU, IP_RE_CONSTANT = 2, 3, 4
IP_SOURCE_ILLUMINATE, IP_SOURCE_THERMAL = 1, 2


class RunesArgs(C.Structure):
    """socgpu_runes_args."""
    _fields_ = [
        ("n_profile", C.c_int), ("n_layer", C.c_int), ("spectrum_name", C.c_char_p), ("i_source", C.c_int),
        ("p_layer", _dp), ("t_layer", _dp), ("mass", _dp), ("density", _dp), ("p_level", _dp), ("t_level", _dp),
        ("gas", _dp * RUNES_N_GAS), ("gas_mix_ratio", C.c_double * RUNES_N_GAS),
        ("has_mix_ratio", C.c_int * RUNES_N_GAS), ("gas_well_mixed", C.c_int * RUNES_N_GAS),
        ("l_invert", C.c_int),
        ("t_ground", _dp), ("l_flux_ground", C.c_int), ("flux_ground", _dp),
        ("cos_zenith_angle", _dp), ("solar_irrad", _dp),
        ("l_grey_albedo", C.c_int), ("grey_albedo", C.c_double), ("albedo_diff", _dp), ("albedo_dir", _dp),
        ("l_tile", C.c_int), ("n_tile", C.c_int), ("l_flux_tile", _ip), ("frac_tile", _dp), ("t_tile", _dp),
        ("flux_tile", _dp), ("albedo_diff_tile", _dp), ("albedo_dir_tile", _dp),
        ("i_scatter_method", C.c_int), ("i_gas_overlap", C.c_int), ("l_rayleigh", C.c_int),
        ("l_mixing_ratio", C.c_int),
        ("l_aerosol_mode", C.c_int), ("n_aer_mode", C.c_int), ("aer_mix_ratio", _dp), ("aer_absorption", _dp),
        ("aer_scattering", _dp), ("aer_asymmetry", _dp),
        ("layer_heat_capacity", _dp), ("precision", C.c_int),
        ("aerosol", _dp * RUNES_N_AER), ("mean_rel_humidity", _dp),
        ("i_cloud_representation", C.c_int), ("i_overlap", C.c_int), ("i_inhom", C.c_int),
        ("i_cloud_entrapment", C.c_int), ("i_mcica_sampling", C.c_int), ("i_st_water", C.c_int),
        ("i_st_ice", C.c_int), ("i_drop_re", C.c_int), ("n_cloud_layer", C.c_int),
        ("cloud_frac", _dp), ("conv_frac", _dp), ("liq_frac", _dp), ("ice_frac", _dp), ("liq_conv_frac", _dp),
        ("ice_conv_frac", _dp), ("liq_mmr", _dp), ("ice_mmr", _dp), ("liq_conv_mmr", _dp), ("ice_conv_mmr", _dp),
        ("liq_dim", _dp), ("ice_dim", _dp), ("liq_rsd", _dp), ("ice_rsd", _dp),
        ("has_liq_dim_constant", C.c_int), ("has_cloud_vertical_decorr", C.c_int),
        ("has_cloud_horizontal_rsd", C.c_int), ("liq_dim_constant", C.c_double),
        ("cloud_vertical_decorr", C.c_double), ("cloud_horizontal_rsd", C.c_double),
        ("rand_seed", _ip), ("mcica_data", C.c_char_p),
        ("i_cnv_water", C.c_int), ("i_cnv_ice", C.c_int), ("liq_conv_dim", _dp), ("ice_conv_dim", _dp),
        ("liq_conv_rsd", _dp), ("ice_conv_rsd", _dp), ("has_liq_conv_dim_constant", C.c_int),
        ("liq_conv_dim_constant", C.c_double), ("has_conv_vertical_decorr", C.c_int),
        ("conv_vertical_decorr", C.c_double),
    ]


class RunesDiag(C.Structure):
    """socgpu_runes_diag."""
    _fields_ = [(n, _dp) for n in ("heating_rate", "flux_up", "flux_down", "flux_direct", "flux_up_surf",
                                   "flux_down_surf", "flux_direct_surf", "flux_up_toa", "flux_down_toa",
                                   "flux_direct_toa")]


class Bound(C.Structure):
    _fields_ = [("zen_0", _dp), ("solar_irrad", _dp), ("rho_alb", _dp), ("t_ground", _dp), ("flux_ground", _dp)]


class Aer(C.Structure):
    _fields_ = [
        ("n_mode", C.c_int), ("mode_mix_ratio", _dp), ("mode_absorption", _dp),
        ("mode_scattering", _dp), ("mode_asymmetry", _dp),
        ("n_aerosol_mr", C.c_int), ("mix_ratio", _dp), ("mr_type_index", _ip), ("mr_source", _ip),
        ("mean_rel_humidity", _dp),
        ("n_opt_level_prsc", _ip), ("n_phase_term_prsc", _ip), ("pressure_prsc", _dp), ("absorption_prsc", _dp),
        ("scattering_prsc", _dp), ("phase_fnc_prsc", _dp),
    ]


class Cld(C.Structure):
    _fields_ = [
        ("n_condensed", C.c_int), ("type_condensed", _ip), ("i_cloud_type", _ip), ("i_condensed_param", _ip),
        ("i_condensed_type", _ip), ("condensed_mix_ratio", _dp), ("condensed_dim_char", _dp),
        ("n_cloud_type", C.c_int), ("w_cloud", _dp), ("frac_cloud", _dp),
        ("n_subcol_gen", C.c_int), ("n_subcol_req", C.c_int), ("c_sub", _dp), ("frac_cloudy", _dp),
        ("n_subcol_cld", _ip), ("subcol_k", _ip), ("first_subcol_k", _ip), ("subcol_reorder", _ip),
        ("dp_corr_strat", C.c_double), ("dp_corr_conv", C.c_double),
    ]


class Radout(C.Structure):
    _fields_ = [
        ("flux_up", _dp), ("flux_down", _dp), ("flux_direct", _dp), ("flux_div", _dp),
        ("heating_rate", _dp), ("flux_up_band", _dp), ("flux_down_band", _dp),
    ]


class BatchItem(C.Structure):
    _fields_ = [
        ("control", C.POINTER(Control)), ("dimen", C.POINTER(Dimen)), ("spectrum", C.c_int32),
        ("atm", C.POINTER(Atm)), ("cld", C.POINTER(Cld)), ("aer", C.POINTER(Aer)), ("bound", C.POINTER(Bound)),
        ("radout", C.POINTER(Radout)),
    ]


class ServerConfig(C.Structure):
    _fields_ = [("device_bytes", C.c_size_t), ("streams", C.c_int), ("max_wave_requests", C.c_int),
                ("small_column_gpoints", C.c_longlong)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("waves", C.c_longlong),
                ("max_wave_requests", C.c_longlong), ("queued", C.c_longlong), ("column_gpoints", C.c_longlong),
                ("device_bytes", C.c_size_t), ("peak_bytes", C.c_size_t), ("max_waves_in_flight", C.c_longlong),
                ("small_waves", C.c_longlong)]


SERVER_PENDING = 100

ABI_FUNCTIONS = (
    "socgpu_abi_version", "socgpu_spectrum_register", "socgpu_spectrum_lookup", "socgpu_spectrum_n_gpoint",
    "socgpu_spectrum_release", "socgpu_radiance_calc", "socgpu_radiance_calc_device", "socgpu_cloud_gen",
    "socgpu_cloud_gen_device", "socgpu_kernel_launch_count", "socgpu_set_device", "socgpu_set_tile_config",
    "socgpu_cloud_gen_device_noalloc", "socgpu_batch_create", "socgpu_batch_run", "socgpu_batch_tune",
    "socgpu_batch_info", "socgpu_batch_destroy", "socgpu_tune_get", "socgpu_tune_set",
    "socgpu_server_create", "socgpu_server_submit", "socgpu_server_wait", "socgpu_server_stats_get",
    "socgpu_server_destroy", "socgpu_spectrum_load", "socgpu_spectrum_load_ext", "socgpu_runes",
    "socgpu_spectrum_k_terms", "socgpu_spectrum_aerosols", "socgpu_spectrum_set_aerosol_parm",
)

_CALC_ARGS = [C.POINTER(Control), C.POINTER(Dimen), C.c_int, C.POINTER(Atm), C.POINTER(Cld), C.POINTER(Aer),
              C.POINTER(Bound), C.POINTER(Radout)]
_GEN_ARGS = [C.c_int] * 11 + [C.c_void_p] + [C.c_void_p] * 8 + [C.c_void_p, C.c_void_p, C.c_int]


def declare(lib: C.CDLL) -> C.CDLL:
    """Attach argument and return types of the ABI to a loaded library."""
    lib.socgpu_abi_version.restype = C.c_int
    lib.socgpu_spectrum_register.argtypes = [C.c_char_p, C.POINTER(SpectrumDesc), C.POINTER(C.c_int), C.c_char_p,
                                             C.c_size_t]
    lib.socgpu_spectrum_lookup.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    lib.socgpu_spectrum_load.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_int), C.c_char_p, C.c_size_t]
    lib.socgpu_spectrum_load_ext.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_int),
                                             C.c_char_p, C.c_size_t]
    lib.socgpu_runes.argtypes = [C.POINTER(RunesArgs), C.POINTER(RunesDiag), C.c_char_p, C.c_size_t]
    lib.socgpu_spectrum_n_gpoint.argtypes = [C.c_int]
    lib.socgpu_spectrum_k_terms.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                            C.POINTER(C.c_int)]
    lib.socgpu_spectrum_aerosols.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                             C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.socgpu_spectrum_set_aerosol_parm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_size_t]
    lib.socgpu_spectrum_release.argtypes = [C.c_int]
    lib.socgpu_radiance_calc.argtypes = _CALC_ARGS + [C.c_char_p, C.c_size_t]
    lib.socgpu_radiance_calc_device.argtypes = _CALC_ARGS + [C.c_void_p, C.c_char_p, C.c_size_t]
    lib.socgpu_cloud_gen.argtypes = _GEN_ARGS + [C.c_char_p, C.c_size_t]
    lib.socgpu_cloud_gen_device.argtypes = _GEN_ARGS + [C.c_void_p, C.c_char_p, C.c_size_t]
    lib.socgpu_cloud_gen_device_noalloc.argtypes = _GEN_ARGS + [C.c_void_p, C.c_char_p, C.c_size_t]
    lib.socgpu_batch_create.argtypes = [C.POINTER(BatchItem), C.c_int, C.POINTER(C.c_void_p), C.c_char_p,
                                        C.c_size_t]
    lib.socgpu_batch_run.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
    lib.socgpu_batch_tune.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_char_p, C.c_size_t]
    lib.socgpu_batch_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_longlong),
                                      C.POINTER(C.c_longlong)]
    lib.socgpu_batch_destroy.argtypes = [C.c_void_p]
    lib.socgpu_tune_get.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int)]
    lib.socgpu_tune_set.argtypes = [C.c_int] * 6
    lib.socgpu_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]
    lib.socgpu_server_submit.argtypes = [C.c_void_p, C.POINTER(BatchItem), C.POINTER(C.c_longlong), C.c_char_p,
                                         C.c_size_t]
    lib.socgpu_server_wait.argtypes = [C.c_void_p, C.c_longlong, C.c_double, C.POINTER(C.c_int),
                                       C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_char_p, C.c_size_t]
    lib.socgpu_server_stats_get.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
    lib.socgpu_server_destroy.argtypes = [C.c_void_p]
    lib.socgpu_kernel_launch_count.restype = C.c_longlong
    lib.socgpu_set_device.argtypes = [C.c_int]
    lib.socgpu_set_tile_config.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
    for name in ABI_FUNCTIONS:
        f = getattr(lib, name)
        if name != "socgpu_kernel_launch_count":
            f.restype = C.c_int
    return lib


def header_functions(header: Path) -> list[str]:
    """Names of the entry points declared in a header (for the export test)."""
    import re
    text = header.read_text()
    return sorted(set(re.findall(r"SOCGPU_API\s+(?:int|long long)\s+(socgpu_\w+)\s*\(", text)))
