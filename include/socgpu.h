/*
 * socgpu.h -- C-ABI of the GB300 two-stream flux path for SOCRATES.
 *
 * This is the drop-in boundary a SOCRATES host program binds to (Fortran
 * through ISO_C_BINDING, Python through ctypes).  Every entry point takes
 * plain pointers and sizes; no CUDA or C++ type crosses the boundary.
 *
 * Conventions (identical to the reference's Fortran):
 *   - Arrays are column-major with the profile index fastest, exactly as the
 *     reference's derived types hold them, e.g. atm%p(nd_profile, nd_layer)
 *     (src/radiance_core/def_atm.F90).  The allocated extent nd_* is passed
 *     separately from the valid extent n_*.
 *   - Level arrays run 0..n_layer (level 0 = top of atmosphere), layer
 *     arrays 1..n_layer (layer i lies between levels i-1 and i).
 *   - Option identifiers carry the reference's rad_pcf values
 *     (src/radiance_core/rad_pcf.F90).  Status codes are the reference's
 *     error codes (rad_pcf.F90:391-405).  No entry point stops the process;
 *     failures return a status and a message.
 *   - All arithmetic on the reference path is FP64.  SOCGPU_PRECISION_FP64
 *     keeps that; SOCGPU_PRECISION_MIXED (no counterpart in the reference)
 *     runs the bulk in FP32.
 */
#ifndef SOCGPU_H
#define SOCGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SOCGPU_API __attribute__((visibility("default")))
#else
#define SOCGPU_API
#endif

#define SOCGPU_ABI_VERSION 7

/* ---- status codes: rad_pcf.F90:391-405 ------------------------------- */
#define SOCGPU_I_NORMAL             0
#define SOCGPU_I_ERR_FATAL          1
#define SOCGPU_I_ABORT_CALCULATION  2
#define SOCGPU_I_ERR_IO             4
#define SOCGPU_I_ERR_RANGE          5
#define SOCGPU_I_ERR_EXIST          6

/* ---- option identifiers (rad_pcf.F90 values) ------------------------- */
#define SOCGPU_IP_SOLAR                 1   /* rad_pcf.F90:602 */
#define SOCGPU_IP_INFRA_RED             2   /* rad_pcf.F90:604 */
#define SOCGPU_IP_TWO_STREAM            1   /* rad_pcf.F90:176 */
/* two-stream schemes, rad_pcf.F90:700-722 */
#define SOCGPU_IP_EDDINGTON             2
#define SOCGPU_IP_DISCRETE_ORD          4
#define SOCGPU_IP_IFM                   5
#define SOCGPU_IP_PIFM85                6
#define SOCGPU_IP_ZDK_FLUX              7
#define SOCGPU_IP_KRSCHG_FLUX           8
#define SOCGPU_IP_COAKLEY_CHYLEK_1      9
#define SOCGPU_IP_COAKLEY_CHYLEK_2     10
#define SOCGPU_IP_MEADOR_WEAVER        11
#define SOCGPU_IP_ELSASSER             12
#define SOCGPU_IP_2S_TEST              14
#define SOCGPU_IP_HEMI_MEAN            15
#define SOCGPU_IP_PIFM80               16
/* scattering treatment, rad_pcf.F90:539-545 */
#define SOCGPU_IP_SCATTER_FULL          1
#define SOCGPU_IP_NO_SCATTER_ABS        2
#define SOCGPU_IP_NO_SCATTER_EXT        3
/* direct-beam optical depth, rad_pcf.F90:553-557 */
#define SOCGPU_IP_DIRECT_NOSCALING      0
#define SOCGPU_IP_DIRECT_DELTA_SCALING  1
#define SOCGPU_IP_DIRECT_CSR_SCALING    2
/* solvers, rad_pcf.F90:566-572 */
#define SOCGPU_IP_SOLVER_NO_SCAT        2
#define SOCGPU_IP_SOLVER_MIX_DIRECT     11   /* two cloud regions (solver_mix_direct.F90) */
#define SOCGPU_IP_SOLVER_HOMOGEN_DIRECT 13
#define SOCGPU_IP_SOLVER_MIX_DIRECT_HOGAN 16 /* two regions, Hogan's form (solver_mix_direct_hogan.F90) */
#define SOCGPU_IP_SOLVER_TRIPLE_HOGAN  17  /* three regions, Hogan's form (solver_triple_hogan.F90) */
/* cloud schemes, rad_pcf.F90:313,322 */
#define SOCGPU_IP_CLOUD_MIX_MAX         2   /* clear and cloudy regions, maximum-random overlap */
#define SOCGPU_IP_CLOUD_MIX_RANDOM      4   /* clear and cloudy regions, random overlap */
#define SOCGPU_IP_CLOUD_TRIPLE          6   /* clear, stratiform and convective regions, maximum-random */
#define SOCGPU_IP_CLOUD_PART_CORR       7   /* clear and cloudy regions, like regions correlated over
                                               dp_corr_strat (rad_pcf.F90:317) */
#define SOCGPU_IP_CLOUD_PART_CORR_CNV   8   /* three regions, stratiform over dp_corr_strat and
                                               convective over dp_corr_conv (rad_pcf.F90:319) */
#define SOCGPU_IP_CLOUD_CLEAR           5
#define SOCGPU_IP_CLOUD_MCICA          10
/* cloud representation, rad_pcf.F90:238-254 */
#define SOCGPU_IP_CLOUD_HOMOGEN         1   /* one cloud type of all components */
#define SOCGPU_IP_CLOUD_ICE_WATER       2
#define SOCGPU_IP_CLOUD_CONV_STRAT      3   /* representations, rad_pcf.F90:238-260 */
#define SOCGPU_IP_CLOUD_CSIW            4
#define SOCGPU_IP_CLOUD_OFF             5
#define SOCGPU_IP_CLOUD_COMBINE_HOMOGEN   6
#define SOCGPU_IP_CLOUD_COMBINE_ICE_WATER 7
#define SOCGPU_IP_CLOUD_SPLIT_HOMOGEN     8
#define SOCGPU_IP_CLOUD_SPLIT_ICE_WATER   9
/* condensate inhomogeneity and cloud entrapment, rad_pcf.F90:267-286 */
#define SOCGPU_IP_MAX_ENTRAPMENT        1
#define SOCGPU_IP_ZERO_ENTRAPMENT       2
#define SOCGPU_IP_HOMOGENEOUS           0
#define SOCGPU_IP_SCALING               1
#define SOCGPU_IP_MCICA                 2
#define SOCGPU_IP_TRIPLECLOUDS_2019     4   /* rad_pcf.F90:286 */
/* droplet effective radius, rad_pcf.F90:356-360 */
#define SOCGPU_IP_RE_EXTERNAL           2
#define SOCGPU_IP_RE_LIU                3
#define SOCGPU_IP_RE_CONSTANT           4
/* cloud types, rad_pcf.F90:332-348: water and ice; stratiform and
   convective; stratiform water and ice, convective water and ice */
#define SOCGPU_IP_CLOUD_TYPE_WATER      1
#define SOCGPU_IP_CLOUD_TYPE_ICE        2
#define SOCGPU_IP_CLOUD_TYPE_STRAT      1
#define SOCGPU_IP_CLOUD_TYPE_CONV       2
#define SOCGPU_IP_CLOUD_TYPE_SW         1
#define SOCGPU_IP_CLOUD_TYPE_SI         2
#define SOCGPU_IP_CLOUD_TYPE_CW         3
#define SOCGPU_IP_CLOUD_TYPE_CI         4
/* condensed components, rad_pcf.F90:187-193: stratiform and convective water and ice */
#define SOCGPU_IP_CLCMP_ST_WATER        1
#define SOCGPU_IP_CLCMP_ST_ICE          2
#define SOCGPU_IP_CLCMP_CNV_WATER       3
#define SOCGPU_IP_CLCMP_CNV_ICE         4
/* condensed phases, rad_pcf.F90:494-496 */
#define SOCGPU_IP_PHASE_WATER           1
#define SOCGPU_IP_PHASE_ICE             2
/* condensed-phase parametrizations, rad_pcf.F90:206,486 */
/* cloud parametrization schemes (rad_pcf.F90:200-209, 447-486) */
#define SOCGPU_IP_SLINGO_SCHRECKER      1   /* droplets: k = q (a1 + a2/re), 1 - w = a3 + a4 re, g = a5 + a6 re */
#define SOCGPU_IP_DROP_PADE_2           5
#define SOCGPU_IP_SLINGO_SCHRECKER_ICE  1   /* ice: the same form in the ice dimension */
#define SOCGPU_IP_ICE_FU_PHF           12   /* Fu's ice fits, one phase-function moment (opt_prop_fu_phf_mod.F90) */
#define SOCGPU_IP_ICE_PADE_2_PHF       20
/* gas overlap, rad_pcf.F90:427 */
#define SOCGPU_IP_OVERLAP_HYBRID        0   /* rad_pcf.F90:423: each band's method from the spectral file */
#define SOCGPU_IP_OVERLAP_RANDOM        2
#define SOCGPU_IP_OVERLAP_K_EQV_SCL     4   /* rad_pcf.F90:432: equivalent extinction of minor gases */
#define SOCGPU_IP_OVERLAP_K_EQV         5   /* rad_pcf.F90:434: solved as K_EQV_SCL */
#define SOCGPU_IP_OVERLAP_K_EQV_MOD     6   /* rad_pcf.F90:436: solved as K_EQV_SCL */
/* k scaling, rad_pcf.F90:412-416 and 509-515 */
#define SOCGPU_IP_SCALE_NULL            0
#define SOCGPU_IP_SCALE_BAND            1
#define SOCGPU_IP_SCALE_TERM            2
#define SOCGPU_IP_SCALE_FNC_NULL        0
#define SOCGPU_IP_SCALE_POWER_LAW       1
#define SOCGPU_IP_SCALE_POWER_QUAD      2
#define SOCGPU_IP_SCALE_DOPPLER_QUAD    3
#define SOCGPU_IP_SCALE_WENYI           4   /* CO2 tables of bands 4 and 6 (scale_absorb.F90:238-281) */
#define SOCGPU_IP_SCALE_LOOKUP          9   /* P/T (and gas-fraction) tables of the '_k' file */
#define SOCGPU_IP_SCALE_T_LOOKUP       10   /* temperature tables of the '_k' file */
/* Rayleigh schemes, rad_pcf.F90:729-731 */
#define SOCGPU_IP_RAYLEIGH_TOTAL        1
/* parametrizations of aerosol species (rad_pcf.F90:22-30) */
#define SOCGPU_IP_AEROSOL_PARAM_DRY       1   /* mass coefficients and an asymmetry */
#define SOCGPU_IP_AEROSOL_PARAM_MOIST     2   /* the same, tabulated in relative humidity */
#define SOCGPU_IP_AEROSOL_UNPARAMETRIZED  3   /* observed optical properties: not supported */
#define SOCGPU_IP_AEROSOL_PARAM_PHF_DRY   4   /* moments of the phase function */
#define SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST 5
/* sources of aerosol mixing ratios (rad_pcf.F90:163-170); the radiatively
   active ones are 0-2, each inactive one is its active one plus 10 */
#define SOCGPU_IP_AERSRC_CUSACK_RON       0
#define SOCGPU_IP_AERSRC_CLASSIC_RON      1
#define SOCGPU_IP_AERSRC_ARCL_RON         2
/* Continuum types (rad_pcf.F90 ip_self_continuum, ip_frn_continuum) */
#define SOCGPU_IP_SELF_CONTINUUM 1
#define SOCGPU_IP_FRN_CONTINUUM  2

/* McICA overlap (socrates_cloud_gen.F90 ioverlap), rad_pcf.F90:294-300 */
#define SOCGPU_IP_MAX_RAND              0
#define SOCGPU_IP_RAND                  1
#define SOCGPU_IP_EXPONENTIAL           2
#define SOCGPU_IP_EXPONENTIAL_RAND      3
/* McICA sampling, def_mcica.F90:22-26 */
#define SOCGPU_IP_MCICA_FULL_SAMPLING    0
#define SOCGPU_IP_MCICA_SINGLE_SAMPLING  1
#define SOCGPU_IP_MCICA_OPTIMAL_SAMPLING 2

/* ---- extensions with no counterpart in the reference ----------------- */
#define SOCGPU_PRECISION_FP64   0   /* every operation in FP64 */
#define SOCGPU_PRECISION_MIXED  1   /* FP32 bulk, stable reformulations */

/* McICA random number generator */
#define SOCGPU_RNG_LCG     0   /* the reference generator, socrates_cloud_gen.F90:48-50 */
#define SOCGPU_RNG_PHILOX  1   /* counter-based Philox4x32-10 keyed by (seed, column, subcolumn, layer) */

/* Limits of the device path. */
#define SOCGPU_MAX_LAYER        512
#define SOCGPU_MAX_BAND          64
#define SOCGPU_MAX_GPOINT      4096
#define SOCGPU_MAX_SPECIES       32
#define SOCGPU_MAX_MODE          16
#define SOCGPU_MAX_SUBCOL        64

/* ---- spectral file ----------------------------------------------------
 * A flat view of the reference's StrSpecData (src/radiance_core/
 * def_spectrum.F90).  Pointers are host memory, Fortran layout, with the
 * nd_* dimensions of the spectrum type.  NULL marks an absent block.    */
typedef struct socgpu_spectrum_desc {
    /* StrSpecDim */
    int nd_band, nd_species, nd_k_term, nd_scale_variable;
    int nd_thermal_coeff, nd_drop_type, nd_ice_type, nd_cloud_parameter;
    /* StrSpecBasic, block 1 */
    int n_band;
    const double *wavelength_short;     /* (nd_band) [m] */
    const double *wavelength_long;      /* (nd_band) [m] */
    /* StrSpecSolar, blocks 2 and 3 */
    const double *solar_flux_band;      /* (nd_band) fraction of the solar constant, or NULL */
    int i_rayleigh_scheme;              /* SOCGPU_IP_RAYLEIGH_TOTAL */
    const double *rayleigh_coeff;       /* (nd_band) [m2/kg], or NULL */
    /* StrSpecGas, blocks 0, 4 and 5 */
    int n_absorb;
    const int    *type_absorb;          /* (nd_species) */
    const int    *n_band_absorb;        /* (nd_band) */
    const int    *index_absorb;         /* (nd_species, nd_band), 1-based species indices */
    const int    *i_band_k;             /* (nd_band, nd_species) */
    const int    *i_scale_k;            /* (nd_band, nd_species) */
    const int    *i_scale_fnc;          /* (nd_band, nd_species) */
    const double *k;                    /* (nd_k_term, nd_band, nd_species) [m2/kg] */
    const double *w;                    /* (nd_k_term, nd_band, nd_species) */
    const double *scale;                /* (nd_scale_variable, nd_k_term, nd_band, nd_species) */
    const double *p_ref;                /* (nd_species, nd_band) [Pa] */
    const double *t_ref;                /* (nd_species, nd_band) [K] */
    const int    *l_doppler;            /* (nd_species) or NULL */
    const double *doppler_cor;          /* (nd_species) or NULL */
    /* StrSpecPlanck, block 6 */
    int n_deg_fit;
    double t_ref_planck;
    const double *thermal_coeff;        /* (0:nd_thermal_coeff-1, nd_band) or NULL */
    /* StrSpecDrop, block 10 */
    const int    *l_drop_type;          /* (nd_drop_type) or NULL: the type is defined */
    const int    *i_drop_parm;          /* (nd_drop_type) scheme of each type, indexed by the
                                           file's type number (read_spectrum.F90 block 10) */
    const double *drop_parm_list;       /* (nd_cloud_parameter, nd_band, nd_drop_type) */
    /* StrSpecIce, block 12 */
    const int    *l_ice_type;           /* (nd_ice_type) or NULL */
    const int    *i_ice_parm;           /* (nd_ice_type) scheme of each type (block 12) */
    const double *ice_parm_list;        /* (nd_cloud_parameter, nd_band, nd_ice_type) */
    /* StrSpecCont, blocks 8 and 9 (NULL n_band_continuum: no continua) */
    int nd_continuum;
    const int    *n_band_continuum;     /* (nd_band) */
    const int    *index_continuum;      /* (nd_band, nd_continuum): SOCGPU_IP_SELF_CONTINUUM / FRN */
    int index_water;                    /* 1-based absorber index of water vapour */
    const int    *i_scale_fnc_cont;     /* (nd_band, nd_continuum) */
    const double *k_cont;               /* (nd_band, nd_continuum) [m5/(kg mol)] */
    const double *scale_cont;           /* (nd_scale_variable, nd_band, nd_continuum) */
    const double *p_ref_cont;           /* (nd_continuum, nd_band) [Pa] */
    const double *t_ref_cont;           /* (nd_continuum, nd_band) [K] */
    /* Lookup-table k scaling, read from the '_k' companion file of block 5
       (read_spectrum.F90:1340-1560; inter_pt_lookup.F90, inter_t_lookup.F90).
       Absorbers with i_scale_fnc SOCGPU_IP_SCALE_LOOKUP take their k from
       k_lookup (or k_lookup_sb when self-broadened), not from k. */
    int n_pre, n_tmp;                   /* P/T table extents (0: no P/T tables) */
    const double *p_lookup;             /* (n_pre) ln(p / Pa), increasing */
    const double *t_lookup;             /* (n_tmp, n_pre) [K], increasing along n_tmp */
    const double *k_lookup;             /* (n_tmp, n_pre, nd_k_term, nd_species, nd_band) [m2/kg] */
    const int    *index_sb;             /* (nd_species) 1-based self-broadened index, 0: none; or NULL */
    int nd_species_sb, n_gas_frac;      /* self-broadened absorbers, gas-fraction table extent */
    const double *gf_lookup;            /* (n_gas_frac) gas fractions, increasing */
    const double *k_lookup_sb;          /* (n_tmp, n_pre, n_gas_frac, nd_k_term, nd_species_sb, nd_band) */
    const double *molar_weight;         /* (nd_species) [g/mol] of each absorber, for self-broadening */
    int nd_t_lookup_gas;                /* temperature-only tables (SOCGPU_IP_SCALE_T_LOOKUP) */
    const int    *n_t_lookup_gas;       /* (nd_species) */
    const double *t_lookup_gas;         /* (nd_t_lookup_gas, nd_species) [K], increasing */
    const double *k_t_lookup_gas;       /* (nd_t_lookup_gas, nd_k_term, nd_species, nd_band) [m2/kg] */
    /* Wen-Yi Zhong's CO2 tables for SOCGPU_IP_SCALE_WENYI (module scale_wenyi);
       the reference compiles them in, here the caller supplies them. */
    int wenyi_n_term4, wenyi_n_term6;   /* third extents of wenyi_gk4 / wenyi_gk6 (0: absent) */
    const double *wenyi_plg;            /* (26) ln(p / 100 Pa) grid */
    const double *wenyi_ttb;            /* (10) temperatures of the band-4 table [K] */
    const double *wenyi_tto;            /* (9) temperatures of the band-6 table [K] */
    const double *wenyi_gk250b;         /* (wenyi_n_term4) band-4 normalisation at 250 K */
    const double *wenyi_gk4;            /* (10, 26, wenyi_n_term4) */
    const double *wenyi_gk6;            /* (9, 26, wenyi_n_term6) */
    /* StrSpecAerosol, block 11 (read_spectrum.F90:2335-2640): the classic
       aerosol species; n_aerosol 0 (or NULL arrays): none */
    int n_aerosol, nd_aerosol_species, nd_humidity, nd_phase_term;
    const int    *type_aerosol;         /* (nd_aerosol_species) type numbers */
    const int    *i_aerosol_parm;       /* (nd_aerosol_species) SOCGPU_IP_AEROSOL_PARAM_* */
    const int    *nhumidity;            /* (nd_aerosol_species) humidities tabulated (moist), 0 (dry) */
    const int    *n_aerosol_phf_term;   /* (nd_aerosol_species) phase-function moments */
    const double *aerosol_humidities;   /* (nd_humidity, nd_aerosol_species) */
    const double *aerosol_abs;          /* (nd_humidity, nd_aerosol_species, nd_band) [m2/kg] */
    const double *aerosol_scat;         /* (nd_humidity, nd_aerosol_species, nd_band) [m2/kg] */
    const double *aerosol_phf;          /* (nd_humidity, nd_phase_term, nd_aerosol_species, nd_band) */
    /* ranges of validity [m] of the droplet and ice parameter sets (blocks 10
       and 12: parm_min_dim, parm_max_dim), indexed like i_drop_parm and
       i_ice_parm; NULL: no limits (set_cld_dim clamps sizes to them) */
    const double *drop_parm_min_dim, *drop_parm_max_dim;
    const double *ice_parm_min_dim, *ice_parm_max_dim;
    /* the gas overlap method each band names (block 4 version 1,
       Sp%Gas%i_overlap, read_spectrum.F90:1012-1016), which a control of
       SOCGPU_IP_OVERLAP_HYBRID takes (radiance_calc.F90:888-893); NULL or 0:
       none named */
    const int *i_overlap;               /* (nd_band) */
} socgpu_spectrum_desc;

typedef int32_t socgpu_spectrum_handle;   /* > 0 when valid */

/* ---- StrCtrl subset (src/radiance_core/def_control.F90) -------------- */
typedef struct socgpu_control {
    int isolir;                 /* SOCGPU_IP_SOLAR | SOCGPU_IP_INFRA_RED */
    int i_angular_integration;  /* SOCGPU_IP_TWO_STREAM only */
    int i_2stream;              /* two-stream scheme */
    int i_scatter_method;       /* SOCGPU_IP_SCATTER_FULL | NO_SCATTER_ABS | NO_SCATTER_EXT */
    int i_solver;               /* SOCGPU_IP_SOLVER_NO_SCAT | SOLVER_HOMOGEN_DIRECT */
    int i_cloud;                /* SOCGPU_IP_CLOUD_CLEAR | SOCGPU_IP_CLOUD_MCICA */
    int i_cloud_representation; /* SOCGPU_IP_CLOUD_ICE_WATER with McICA */
    int i_gas_overlap;          /* SOCGPU_IP_OVERLAP_RANDOM | K_EQV_SCL (K_EQV, K_EQV_MOD alike) | HYBRID
                                   (the method the spectrum's bands name; the bands of the call must agree) */
    int i_direct_tau;           /* SOCGPU_IP_DIRECT_DELTA_SCALING (default) | NOSCALING; CSR_SCALING refused */
    int l_rescale;              /* delta-rescaling of tau, omega and the phase function */
    int n_order_forward;        /* order of the forward-scattering term (2: f = g^2) */
    int l_ir_source_quad;       /* quadratic IR source */
    int l_rayleigh;
    int l_gas;
    int l_aerosol_mode;         /* modal (UKCA-style) aerosol optics */
    int l_flux_div;             /* accumulate the flux divergence per k-term */
    int first_band, last_band;  /* 1-based, inclusive */
    const double *weight_band;  /* (n_band) or NULL (all 1); device memory for
                                   socgpu_radiance_calc_device */
    int precision;              /* SOCGPU_PRECISION_* (extension) */
    int l_continuum;            /* water-vapour continuum absorption (blocks 8 and 9) */
    int l_mixing_ratio;         /* gas amounts per unit mass of dry air (foreign continuum) */
    int l_grey_single;          /* k_eqv_scl, infra-red: single-term minor gases as grey absorbers */
    int l_aerosol;              /* classic aerosol species of the spectral file (block 11) */
    int l_henyey_greenstein_pf; /* classic aerosol: phase-function moments from the asymmetry */
} socgpu_control;

/* ---- StrDim subset (src/radiance_core/def_dimen.F90) ----------------- */
typedef struct socgpu_dimen {
    int nd_profile, nd_layer;
    int id_cloud_top;           /* first layer that may hold cloud (1-based) */
    int nd_aerosol_mode;
    int nd_cloud_component, nd_cloud_type;
    int nd_subcol_gen, nd_subcol_req;
    int nd_aerosol_mr;          /* third extent of socgpu_aer.mix_ratio */
    /* extents of the prescribed aerosol optical properties (def_dimen.F90
       nd_profile_aerosol_prsc, nd_opt_level_aerosol_prsc,
       nd_phf_term_aerosol_prsc) */
    int nd_profile_aerosol_prsc, nd_opt_level_aerosol_prsc, nd_phf_term_aerosol_prsc;
} socgpu_dimen;

/* ---- StrAtm (src/radiance_core/def_atm.F90) --------------------------- */
typedef struct socgpu_atm {
    int n_profile, n_layer;
    const double *p;             /* (nd_profile, nd_layer) [Pa] */
    const double *t;             /* (nd_profile, nd_layer) [K] */
    const double *p_level;       /* (nd_profile, 0:nd_layer) [Pa] */
    const double *t_level;       /* (nd_profile, 0:nd_layer) [K] */
    const double *mass;          /* (nd_profile, nd_layer) [kg/m2] */
    const double *gas_mix_ratio; /* (nd_profile, nd_layer, nd_species) [kg/kg] */
    const double *density;       /* (nd_profile, nd_layer) [kg/m3]; needed with l_continuum */
} socgpu_atm;

/* ---- StrBound (src/radiance_core/def_bound.F90) ----------------------- */
typedef struct socgpu_bound {
    const double *zen_0;         /* (nd_profile) secant of the solar zenith angle */
    const double *solar_irrad;   /* (nd_profile) [W/m2] */
    const double *rho_alb;       /* (nd_profile, 2, nd_band): diffuse (1) and direct (2) albedo */
    const double *t_ground;      /* (nd_profile) [K] */
    /* (nd_profile, nd_band) [W/m2] or NULL: the surface's Planck flux in each
       band in place of that of t_ground (planck%flux_ground of
       diff_planck_source_mod.F90:123-135, l_flux_ground and surface tiles) */
    const double *flux_ground;
} socgpu_bound;

/* ---- StrAer modal part (src/radiance_core/def_aer.F90:36-44) ---------- */
typedef struct socgpu_aer {
    int n_mode;
    const double *mode_mix_ratio;   /* (nd_profile, nd_layer, nd_aerosol_mode) */
    const double *mode_absorption;  /* (nd_profile, nd_layer, nd_aerosol_mode, nd_band) [m2/kg] */
    const double *mode_scattering;  /* same */
    const double *mode_asymmetry;   /* same */
    /* classic aerosol (def_aer.F90:26-34), with control.l_aerosol: mixing
       ratios of the spectral file's species, and the layers' mean relative
       humidity for moist species */
    int n_aerosol_mr;
    const double *mix_ratio;         /* (nd_profile, nd_layer, nd_aerosol_mr) [kg/kg] */
    const int    *mr_type_index;     /* (nd_aerosol_mr) 1-based species of the spectral file */
    const int    *mr_source;         /* (nd_aerosol_mr) SOCGPU_IP_AERSRC_*: only the active ones count */
    const double *mean_rel_humidity; /* (nd_profile, nd_layer) in [0, 1], or NULL without moist species */
    /* prescribed optical properties (def_aer.F90:46-60) of the species whose
       parametrization in the spectrum is SOCGPU_IP_AEROSOL_UNPARAMETRIZED
       (l_run_cdf's overlay of observed properties): per species, values on
       its own pressure levels (ascending), fitted by cubic splines in
       pressure and evaluated at the layer pressures (prsc_opt_prop.F90,
       prsc_gather_spline.F90); absorption and scattering are volume
       coefficients [1/m], divided by atm.density.  Zero outside the levels. */
    const int    *n_opt_level_prsc;  /* (nd_aerosol_species) levels of each species (host array) */
    const int    *n_phase_term_prsc; /* (nd_aerosol_species) phase-function moments given (host array) */
    const double *pressure_prsc;     /* (nd_profile_aerosol_prsc, nd_opt_level_aerosol_prsc, nd_aerosol_species) [Pa] */
    const double *absorption_prsc;   /* (nd_profile_aerosol_prsc, nd_opt_level_aerosol_prsc, nd_aerosol_species, nd_band) */
    const double *scattering_prsc;   /* same */
    const double *phase_fnc_prsc;    /* (nd_profile_aerosol_prsc, nd_opt_level_aerosol_prsc, nd_phf_term_aerosol_prsc,
                                         nd_aerosol_species, nd_band) */
} socgpu_aer;

/* ---- StrCld with the McICA state (def_cld.F90, def_mcica.F90) --------
 * Cloudy arrays span layers id_cloud_top..nd_layer.  The McICA arrays are
 * what set_cld_mcica (socrates_set_cld_mcica.F90:82-228) leaves in cld.   */
typedef struct socgpu_cld {
    int n_condensed;
    const int *type_condensed;        /* (nd_cloud_component) ip_clcmp_* */
    const int *i_cloud_type;          /* (nd_cloud_component) cloud type of each component */
    const int *i_condensed_param;     /* (nd_cloud_component) parametrization: droplets
                                         SOCGPU_IP_SLINGO_SCHRECKER or _DROP_PADE_2; ice
                                         SOCGPU_IP_SLINGO_SCHRECKER_ICE, _ICE_FU_PHF or
                                         _ICE_PADE_2_PHF; the scheme of the chosen type */
    const int *i_condensed_type;      /* (nd_cloud_component) 1-based drop type (water) or ice type (ice)
                                         in the spectrum: the parameter set parm_list(:, band, type) */
    const double *condensed_mix_ratio;/* (nd_profile, id_ct:nd_layer, nd_cloud_component), in-cloud */
    const double *condensed_dim_char; /* same layout [m] */
    int n_cloud_type;
    const double *w_cloud;            /* (nd_profile, id_ct:nd_layer) cloud fraction */
    const double *frac_cloud;         /* (nd_profile, id_ct:nd_layer, nd_cloud_type), normalised */
    /* McICA */
    int n_subcol_gen, n_subcol_req;
    const double *c_sub;              /* (nd_profile, id_ct:nd_layer, nd_subcol_gen) scaling of cloud water per subcolumn */
    const double *frac_cloudy;        /* (nd_profile) */
    const int *n_subcol_cld;          /* (nd_profile) or NULL.  NULL: c_sub is the filled array that
                                         set_cld_mcica leaves (socrates_set_cld_mcica.F90:206-220).
                                         Non-NULL: c_sub is cloud_gen's compacted output and
                                         subcolumns n_subcol_cld+1..min(n_subcol_req, n_subcol_gen)
                                         read cloudy subcolumn ((j-1) mod n_subcol_cld)+1, which is
                                         what the fill step copies there. */
    const int *subcol_k;              /* (nd_band, nd_k_term) of the spectrum */
    const int *first_subcol_k;        /* (nd_band, nd_k_term+1) of the spectrum */
    const int *subcol_reorder;        /* (nd_subcol_req) */
    /* pressure scales [Pa] over which like stratiform and like convective
       regions decorrelate under SOCGPU_IP_CLOUD_PART_CORR(_CNV)
       (overlap_coupled.F90:209-236) */
    double dp_corr_strat, dp_corr_conv;
} socgpu_cld;

/* ---- StrOut subset (src/radiance_core/def_out.F90), one channel ------ */
typedef struct socgpu_radout {
    double *flux_up;        /* (nd_profile, 0:nd_layer) */
    double *flux_down;      /* (nd_profile, 0:nd_layer), total (direct+diffuse) in the SW */
    double *flux_direct;    /* (nd_profile, 0:nd_layer) SW only, else may be NULL */
    double *flux_div;       /* (nd_profile, nd_layer) when control.l_flux_div, else NULL */
    double *heating_rate;   /* (nd_profile, nd_layer) [K/day] or NULL (extension) */
    double *flux_up_band;   /* (nd_profile, 0:nd_layer, nd_band) or NULL */
    double *flux_down_band; /* (nd_profile, 0:nd_layer, nd_band) or NULL */
} socgpu_radout;

/* ---- entry points ------------------------------------------------------ */

/* Read a spectral file in the reference's text format and register it
 * under `name` (the file-reading half of set_spectrum,
 * src/interface_core/socrates_set_spectrum.F90:90-121; record layouts of
 * src/radiance_core/read_spectrum.F90).  Blocks 0-6, 8, 9, 13 and the
 * Pade cloud blocks 10/12 are read, with the lookup tables of block 5 from
 * the '_k' file beside it (path + "_k"). */
SOCGPU_API int socgpu_spectrum_load(const char *name, const char *path, socgpu_spectrum_handle *handle,
                                    char *msg, size_t msg_len);
/* As socgpu_spectrum_load, with the lookup tables of block 5 read from k_path
   (NULL: path + "_k", read_spectrum.F90:1420-1560) and Wen-Yi Zhong's CO2
   and O3 tables read from wenyi_path, their data file (the reference
   compiles the tables in, module scale_wenyi; socrates_gb300/wenyi.py
   writes the data file from a SOCRATES source tree once; NULL: none, and
   spectra that scale with them are rejected when registered). */
SOCGPU_API int socgpu_spectrum_load_ext(const char *name, const char *path, const char *k_path,
                                        const char *wenyi_path, socgpu_spectrum_handle *handle, char *msg,
                                        size_t msg_len);

/* ABI version of the loaded library (compare with SOCGPU_ABI_VERSION). */
SOCGPU_API int socgpu_abi_version(void);

/* Register a spectral file under a name and keep its tables resident on the
 * device.  Replaces socrates_set_spectrum's cache by name
 * (src/interface_core/socrates_set_spectrum.F90:20-23,90-121): registering
 * a name that already exists returns the existing handle. */
SOCGPU_API int socgpu_spectrum_register(const char *name, const socgpu_spectrum_desc *desc,
                             socgpu_spectrum_handle *handle, char *msg, size_t msg_len);
/* Look a registered spectrum up by name; SOCGPU_I_ERR_EXIST if absent. */
SOCGPU_API int socgpu_spectrum_lookup(const char *name, socgpu_spectrum_handle *handle);
/* Number of g-points (k-term products over the bands) of a spectrum. */
SOCGPU_API int socgpu_spectrum_n_gpoint(socgpu_spectrum_handle handle);
/* Release a spectrum and its device tables. */
SOCGPU_API int socgpu_spectrum_release(socgpu_spectrum_handle handle);
/* The k-term counts set_cld_mcica reads from the spectrum to lay out the
 * McICA sampling (socrates_set_cld_mcica.F90:106-139): the band count,
 * nd_k_term (the leading extent of subcol_k and first_subcol_k) and, for
 * each band, the k-terms of its first absorber (0 without absorbers);
 * n_k_major has room for n_band_max entries.  Any pointer may be NULL. */
SOCGPU_API int socgpu_spectrum_k_terms(socgpu_spectrum_handle handle, int n_band_max, int *n_band, int *nd_k_term,
                                       int *n_k_major);
/* The classic aerosol species of a spectrum (block 11 with the list of
 * block 0): their count and, for up to n_max species, type numbers,
 * parametrizations (SOCGPU_IP_AEROSOL_PARAM_* or _UNPARAMETRIZED) and
 * tabulated humidities.  Any array pointer may be NULL. */
SOCGPU_API int socgpu_spectrum_aerosols(socgpu_spectrum_handle handle, int n_max, int *n_aerosol,
                                        int *type_aerosol, int *i_aerosol_parm, int *nhumidity);
/* Sets the parametrization of species `species` (1-based) of a registered
 * spectrum, as l_run_cdf does when it overlays observed optical properties
 * (input_aerosol_cdf.f:102-143): SOCGPU_IP_AEROSOL_UNPARAMETRIZED (the
 * species then takes socgpu_aer's prescribed properties) or the species'
 * parametrization in its spectral file.  Calls already running keep the
 * value they read; do not change it while another thread submits work that
 * uses the spectrum. */
SOCGPU_API int socgpu_spectrum_set_aerosol_parm(socgpu_spectrum_handle handle, int species, int parm, char *msg,
                                                size_t msg_len);

/* Replaces radiance_calc (src/radiance_core/radiance_calc.F90:16) for the
 * two-stream clear-sky and McICA paths.  All pointers are host memory; the
 * call copies inputs to the device, runs the fused kernels and copies the
 * outputs back before it returns.  Re-entrant: each host thread has its own
 * stream and device workspace. */
SOCGPU_API int socgpu_radiance_calc(const socgpu_control *control, const socgpu_dimen *dimen,
                         socgpu_spectrum_handle spectrum, const socgpu_atm *atm,
                         const socgpu_cld *cld, const socgpu_aer *aer,
                         const socgpu_bound *bound, socgpu_radout *radout,
                         char *msg, size_t msg_len);

/* Same computation with every array pointer in device memory (Fortran
 * layout, the given nd_* extents).  Enqueued on `stream` (a cudaStream_t,
 * NULL for the legacy default stream); returns once the work is enqueued. */
SOCGPU_API int socgpu_radiance_calc_device(const socgpu_control *control, const socgpu_dimen *dimen,
                                socgpu_spectrum_handle spectrum, const socgpu_atm *atm,
                                const socgpu_cld *cld, const socgpu_aer *aer,
                                const socgpu_bound *bound, socgpu_radout *radout,
                                void *stream, char *msg, size_t msg_len);

/* Replaces cloud_gen (src/interface_core/socrates_cloud_gen.F90:8-470):
 * stochastic McICA subcolumns.  Arguments keep the reference's meaning;
 * il1..il2 are 1-based columns, cloud arrays span cloud_top..nd_layer.
 * rng selects the reference LCG or the counter-based Philox stream.
 * Host pointers; synchronous. */
SOCGPU_API int socgpu_cloud_gen(int nd_layer, int cloud_top, int n_layer, int nd_profile,
                     int il1, int il2, int n_subcol, int n1, int n2,
                     int ipph, int ioverlap, const int *rand_seed,
                     const double *rlc_cf, const double *rlc_cw,
                     const double *sigma_qcw, const double *avg_cf,
                     const double *c_cloud, const double *c_ratio,
                     const double *zf, const double *xcw,
                     int *n_subcol_cld, double *c_sub, int rng,
                     char *msg, size_t msg_len);

/* Device-pointer variant of socgpu_cloud_gen, enqueued on `stream`. */
SOCGPU_API int socgpu_cloud_gen_device(int nd_layer, int cloud_top, int n_layer, int nd_profile,
                            int il1, int il2, int n_subcol, int n1, int n2,
                            int ipph, int ioverlap, const int *rand_seed,
                            const double *rlc_cf, const double *rlc_cw,
                            const double *sigma_qcw, const double *avg_cf,
                            const double *c_cloud, const double *c_ratio,
                            const double *zf, const double *xcw,
                            int *n_subcol_cld, double *c_sub, int rng,
                            void *stream, char *msg, size_t msg_len);

/* Most cloud layers (n_layer - cloud_top + 1) socgpu_cloud_gen_device_noalloc
 * accepts: its scratch is a fixed array of 2 * 1024 + 2 ints (8 KB) in the
 * library's device memory. */
#define SOCGPU_NOALLOC_MAX_CLOUD_LAYERS 1024

/* Allocation-free variant of socgpu_cloud_gen_device (extension: no
 * counterpart in the reference, whose cloud_gen keeps its work in automatic
 * arrays sized on every call, src/interface_core/socrates_cloud_gen.F90:
 * 108-138).  Same arguments, same results bit for bit.  It makes no
 * device allocation and no free, for callers that hold a fixed device-memory
 * budget or whose streams must not meet the device-wide synchronisation of a
 * free: its scratch (per-layer cloud flags and the batch's cloud layer range)
 * is a fixed array in the library's device memory.
 * - The first call on each device looks up that array's address; make it
 *   once at set-up, outside any time-critical region.  The address is kept
 *   for the life of the device's primary context: a caller that destroys
 *   that context (cudaDeviceReset) must not call this entry point again in
 *   the same process.
 * - n_layer - cloud_top + 1 above SOCGPU_NOALLOC_MAX_CLOUD_LAYERS is
 *   rejected with SOCGPU_I_ERR_RANGE and a message; nothing is enqueued.
 * - Every call clears the flags it uses on `stream` before use; nothing has to
 *   be zeroed by the caller.
 * - All calls on one device share the scratch: calls that overlap in time
 *   (other streams or host threads, not ordered by the caller) race on it
 *   and give wrong subcolumns.  Serialise them on one stream. */
SOCGPU_API int socgpu_cloud_gen_device_noalloc(int nd_layer, int cloud_top, int n_layer, int nd_profile,
                            int il1, int il2, int n_subcol, int n1, int n2,
                            int ipph, int ioverlap, const int *rand_seed,
                            const double *rlc_cf, const double *rlc_cw,
                            const double *sigma_qcw, const double *avg_cf,
                            const double *c_cloud, const double *c_ratio,
                            const double *zf, const double *xcw,
                            int *n_subcol_cld, double *c_sub, int rng,
                            void *stream, char *msg, size_t msg_len);

/* ---- runes: the model-facing interface ---------------------------------
 * socgpu_runes replaces runes (src/interface_core/socrates_runes.F90:47-1079)
 * for clear-sky calls: set_control's defaults (socrates_set_control.F90:
 * 232-300), the absorbers of the spectrum filled from profiles or
 * well-mixed values (socrates_set_atm.F90:535-622), the surface from a grey
 * or per-band albedo, per-band emission and tiles (socrates_set_bound.F90,
 * diff_planck_source_mod.F90:123-190), and the diagnostics of
 * socrates_set_diag.F90:140-220.  Arrays have the profile index fastest. */
#define SOCGPU_IP_SOURCE_ILLUMINATE 1   /* socrates_runes.F90: the solar source */
#define SOCGPU_IP_SOURCE_THERMAL    2   /* the thermal source */
#define SOCGPU_RUNES_N_GAS         80   /* gas identifiers 1..79 of gas_list_pcf.F90 */
#define SOCGPU_RUNES_N_AER         33   /* aerosol types 1..32 of rad_pcf.F90 */

typedef struct socgpu_runes_args {
    int n_profile, n_layer;
    const char *spectrum_name;          /* registered or loaded under this name (set_spectrum) */
    int i_source;                       /* SOCGPU_IP_SOURCE_ILLUMINATE | SOCGPU_IP_SOURCE_THERMAL */
    /* atmosphere: (n_profile, n_layer) and (n_profile, 0:n_layer) */
    const double *p_layer, *t_layer, *mass, *density, *p_level, *t_level;
    /* absorbers by gas identifier (the <gas>, <gas>_mix_ratio and
       l_<gas>_well_mixed arguments): a profile (n_profile, n_layer), or the
       well-mixed value where there is no profile or gas_well_mixed is set
       with has_mix_ratio; anything else is absent */
    const double *gas[SOCGPU_RUNES_N_GAS];
    double gas_mix_ratio[SOCGPU_RUNES_N_GAS];
    int has_mix_ratio[SOCGPU_RUNES_N_GAS];
    int gas_well_mixed[SOCGPU_RUNES_N_GAS];
    int l_invert;                       /* vertical arrays given surface first */
    /* surface */
    const double *t_ground;             /* (n_profile) [K] */
    int l_flux_ground;
    const double *flux_ground;          /* (n_profile, n_band) surface emission per band [W/m2] */
    const double *cos_zenith_angle, *solar_irrad;   /* (n_profile) */
    int l_grey_albedo;
    double grey_albedo;
    const double *albedo_diff, *albedo_dir;         /* (n_profile, n_band), when not grey */
    int l_tile, n_tile;
    const int *l_flux_tile;             /* (n_tile): the tile's emission is given */
    const double *frac_tile, *t_tile;   /* (n_profile, n_tile) */
    const double *flux_tile;            /* (n_profile, n_tile, n_band) [W/m2] */
    const double *albedo_diff_tile, *albedo_dir_tile;   /* (n_profile, n_tile, n_band) or NULL */
    /* options; 0 selects set_control's default */
    int i_scatter_method, i_gas_overlap;
    int l_rayleigh, l_mixing_ratio;
    /* modal aerosol optical properties */
    int l_aerosol_mode, n_aer_mode;
    const double *aer_mix_ratio;        /* (n_profile, n_layer, n_aer_mode) */
    const double *aer_absorption, *aer_scattering, *aer_asymmetry;  /* (n_profile, n_layer, n_aer_mode, n_band) */
    const double *layer_heat_capacity;  /* (n_profile, n_layer) [J/(m2 K)] or NULL */
    int precision;                      /* SOCGPU_PRECISION_* */
    /* classic aerosol species of the spectral file (set_aer,
       socrates_set_aer.F90:190-290): the mixing ratios (n_profile, n_layer)
       of each aerosol type, indexed by the type number of rad_pcf.F90
       (1 water soluble, 2 dust-like, 3 oceanic, 4 soot, ... 32 two-bin dust
       2); NULL where the runes flag l_<species> is off, and the species is
       then radiatively inactive.  Moist species need mean_rel_humidity. */
    const double *aerosol[SOCGPU_RUNES_N_AER];
    const double *mean_rel_humidity;    /* (n_profile, n_layer) in [0, 1) */
    /* clouds (set_control's cloud options, set_cld, set_cld_dim,
       set_cld_mcica); 0 selects set_control's default */
    int i_cloud_representation;         /* 0 (off), SOCGPU_IP_CLOUD_HOMOGEN, _ICE_WATER, _COMBINE_HOMOGEN,
                                           _COMBINE_ICE_WATER; three regions: _CONV_STRAT, _CSIW,
                                           _SPLIT_HOMOGEN, _SPLIT_ICE_WATER */
    int i_overlap;                      /* SOCGPU_IP_MAX_RAND (0, the default), SOCGPU_IP_RAND,
                                           SOCGPU_IP_EXPONENTIAL_RAND (McICA, or like regions correlated
                                           over cloud_vertical_decorr / conv_vertical_decorr) */
    int i_inhom;                        /* SOCGPU_IP_HOMOGENEOUS, SOCGPU_IP_SCALING, SOCGPU_IP_MCICA,
                                           SOCGPU_IP_TRIPLECLOUDS_2019 (the split representations'
                                           thin and thick parts from the condensate RSD) */
    int i_cloud_entrapment;             /* SOCGPU_IP_ZERO_ENTRAPMENT (default: Hogan's solver) or
                                           SOCGPU_IP_MAX_ENTRAPMENT (solver_mix_direct) */
    int i_mcica_sampling;               /* SOCGPU_IP_MCICA_*_SAMPLING; -1 selects the default, optimal */
    int i_st_water, i_st_ice;           /* droplet and ice types of the spectral file */
    int i_drop_re;                      /* SOCGPU_IP_RE_EXTERNAL (default) or SOCGPU_IP_RE_CONSTANT */
    int n_cloud_layer;                  /* 0: any layer may be cloudy; else only the lowest n_cloud_layer */
    /* (n_profile, n_layer) grid-box fields; conv_* and *_conv_* combine with
       the stratiform ones under the combine representations */
    const double *cloud_frac, *conv_frac, *liq_frac, *ice_frac, *liq_conv_frac, *ice_conv_frac;
    const double *liq_mmr, *ice_mmr, *liq_conv_mmr, *ice_conv_mmr;
    const double *liq_dim, *ice_dim;    /* effective dimensions [m]; NULL: set_cld_dim's parametrizations */
    const double *liq_rsd, *ice_rsd;    /* relative standard deviations of the condensate */
    int has_liq_dim_constant, has_cloud_vertical_decorr, has_cloud_horizontal_rsd;
    double liq_dim_constant;            /* [m], with SOCGPU_IP_RE_CONSTANT */
    double cloud_vertical_decorr;       /* decorrelation pressure scale [Pa] of the McICA generator and of
                                           like stratiform regions */
    double cloud_horizontal_rsd;        /* condensate RSD where liq_rsd / ice_rsd are NULL */
    const int *rand_seed;               /* (n_profile) McICA seeds; NULL: 10 + profile */
    const char *mcica_data;             /* path of the McICA data file (with SOCGPU_IP_MCICA) */
    /* separate convective cloud (SOCGPU_IP_CLOUD_CONV_STRAT, _CSIW,
       _SPLIT_HOMOGEN, _SPLIT_ICE_WATER): the convective droplet and ice
       types, and the convective sizes and RSDs (set_cld_dim's liq_conv_dim,
       ice_conv_dim, liq_conv_dim_constant; set_cld's liq_conv_rsd,
       ice_conv_rsd).  The split representations size and bound their
       convective (optically thick) part by the stratiform arguments. */
    int i_cnv_water, i_cnv_ice;
    const double *liq_conv_dim, *ice_conv_dim;  /* (n_profile, n_layer) [m] or NULL */
    const double *liq_conv_rsd, *ice_conv_rsd;  /* (n_profile, n_layer) or NULL */
    int has_liq_conv_dim_constant;
    double liq_conv_dim_constant;       /* [m], with SOCGPU_IP_RE_CONSTANT */
    /* the pressure scale [Pa] over which like convective regions decorrelate
       under exponential-random overlap (set_cld's conv_vertical_decorr; the
       stratiform scale is cloud_vertical_decorr) */
    int has_conv_vertical_decorr;
    double conv_vertical_decorr;
} socgpu_runes_args;

/* StrDiag (socrates_def_diag.F90): NULL members are not filled. */
typedef struct socgpu_runes_diag {
    double *heating_rate;   /* (n_profile, n_layer): [K/s] with layer_heat_capacity, else the
                               layer's flux divergence [W/m2] */
    double *flux_up, *flux_down, *flux_direct;                   /* (n_profile, 0:n_layer) */
    double *flux_up_surf, *flux_down_surf, *flux_direct_surf;    /* (n_profile) */
    double *flux_up_toa, *flux_down_toa, *flux_direct_toa;       /* (n_profile) */
} socgpu_runes_diag;

/* runes (socrates_runes.F90:47) on the GPU: maps the arguments, calls
 * socgpu_radiance_calc with host arrays and fills the diagnostics.  Clouds
 * of one homogeneous type or of separate water and ice types (and their
 * combinations with convective cloud) run in two regions with maximum-random,
 * random or exponential-random overlap, or with McICA subcolumns; the
 * representations with separate convective cloud run in three regions
 * (clear, stratiform and convective) with maximum-random or
 * exponential-random overlap and Hogan's solver. */
SOCGPU_API int socgpu_runes(const socgpu_runes_args *args, socgpu_runes_diag *diag, char *msg, size_t msg_len);

/* ---- multi-batch launches (extension) -----------------------------------
 * Many column batches of different layer counts, spectra, options and
 * precision in one replay.  The reference has no counterpart: its callers
 * call radiance_calc once per batch (src/radiance_core/radiance_calc.F90:16),
 * which socgpu_radiance_calc_device mirrors.  Every pointer of an item is
 * device memory and must stay valid while the batch exists; the structs
 * themselves are read at creation.  The batches are grouped into kernel
 * classes (precision, mode, tile), each class runs as one persistent launch
 * over all its columns, and the launches are captured in one CUDA graph. */
typedef struct socgpu_batch_item {
    const socgpu_control *control;
    const socgpu_dimen *dimen;
    socgpu_spectrum_handle spectrum;
    const socgpu_atm *atm;
    const socgpu_cld *cld;
    const socgpu_aer *aer;
    const socgpu_bound *bound;
    socgpu_radout *radout;
} socgpu_batch_item;

typedef struct socgpu_batch_s *socgpu_batch;

/* Validate every item (the checks of socgpu_radiance_calc), group, prepare
 * and capture.  On error, msg names the failing item. */
SOCGPU_API int socgpu_batch_create(const socgpu_batch_item *items, int n_items, socgpu_batch *batch,
                                   char *msg, size_t msg_len);

/* Replay all batches on `stream` (one graph launch). */
SOCGPU_API int socgpu_batch_run(socgpu_batch batch, void *stream, char *msg, size_t msg_len);

/* Autotuner: for every (precision, mode, layer count) of the batch, time
 * each built tile (lanes per solve x smallest covering chunk x 4 or 8
 * warps) on the batch's own data, `reps` timed launches each (<1: 3), keep
 * the fastest in the library's tile table (used from then on by every entry
 * point, unless socgpu_set_tile_config overrides it) and recapture.  The
 * outputs are overwritten. */
SOCGPU_API int socgpu_batch_tune(socgpu_batch batch, void *stream, int reps, char *msg, size_t msg_len);

/* Kernel classes, columns and column x g-points of a batch. */
SOCGPU_API int socgpu_batch_info(socgpu_batch batch, int *n_groups, long long *n_columns,
                                 long long *n_column_gpoints);

SOCGPU_API int socgpu_batch_destroy(socgpu_batch batch);

/* The tile table (extension): read or set the entry for (precision, mode
 * 0 lwns / 1 full / 2 mcica, n_layer); lanes_per_solve 0 removes it.  Lets
 * a caller save the tuner's choices and restore them in a later process.
 * lanes_per_solve 1 is the phased kernel (modes 0 and 1, up to 256 layers);
 * its layers_per_lane is the number of k-terms solved per batch (1..32) and
 * its warps_per_cta at least 2. */
SOCGPU_API int socgpu_tune_get(int precision, int mode, int n_layer, int *lanes_per_solve,
                               int *layers_per_lane, int *warps_per_cta);
SOCGPU_API int socgpu_tune_set(int precision, int mode, int n_layer, int lanes_per_solve,
                               int layers_per_lane, int warps_per_cta);

/* ---- request server (extension) -----------------------------------------
 * Continuous batching of radiance_calc requests with host arrays.  The
 * reference has no counterpart: its callers call radiance_calc
 * (src/radiance_core/radiance_calc.F90:16) synchronously, once per batch of
 * columns, as socgpu_radiance_calc does.
 *
 * Every request's inputs and outputs take one block of a device arena of
 * device_bytes while the request is in flight.  A scheduler thread admits
 * queued requests in arrival order while their blocks fit (admission by free
 * device memory) and launches them as one wave on a free stream slot: copy
 * in, one persistent batched launch per kernel class, copy out.  Up to
 * `streams` waves run at once, so new arrivals are admitted as soon as a slot
 * and memory free up, and their work overlaps on the device.  Host arrays
 * (and the option arrays the structs point at) must stay valid until
 * socgpu_server_wait returns for the request.  Page-locked host memory lets
 * the copies run asynchronously. */
typedef struct socgpu_server_config {
    size_t device_bytes;        /* arena for request data; 0: half of the free device memory */
    int streams;                /* waves in flight; 0: 4 */
    int max_wave_requests;      /* requests per wave; 0: 256 */
    /* Requests of at most this many column x g-points are "small": they are
       waved apart from larger ones, on high-priority streams (half of the
       streams, at least one when there are two or more), so that a large
       request in flight does not hold them back; the low-priority streams
       take small requests only while no large request waits or runs.
       0: 131072. */
    long long small_column_gpoints;
} socgpu_server_config;

typedef struct socgpu_server_stats {
    long long submitted, completed, waves, max_wave_requests, queued;
    long long column_gpoints;   /* of the requests completed without error */
    size_t device_bytes, peak_bytes;
    long long max_waves_in_flight;   /* most waves on the device at one time */
    long long small_waves;           /* waves of small requests */
} socgpu_server_stats;

/* A request: the arguments of socgpu_radiance_calc, host pointers. */
typedef socgpu_batch_item socgpu_request;
typedef struct socgpu_server_s *socgpu_server;

/* socgpu_server_wait: the request did not finish within the timeout. */
#define SOCGPU_SERVER_PENDING 100

SOCGPU_API int socgpu_server_create(const socgpu_server_config *config, socgpu_server *server,
                                    char *msg, size_t msg_len);
/* Validate (the checks of socgpu_radiance_calc) and queue; returns at once.
 * A request larger than the arena is rejected with SOCGPU_I_ERR_RANGE. */
SOCGPU_API int socgpu_server_submit(socgpu_server server, const socgpu_request *request, long long *ticket,
                                    char *msg, size_t msg_len);
/* Block until the request is done (timeout_s < 0: no limit); *status is the
 * request's own status (msg its message), *queue_ms the time from submit to
 * launch and *latency_ms from submit to completion.  The ticket is then
 * released. */
SOCGPU_API int socgpu_server_wait(socgpu_server server, long long ticket, double timeout_s, int *status,
                                  double *queue_ms, double *latency_ms, char *msg, size_t msg_len);
SOCGPU_API int socgpu_server_stats_get(socgpu_server server, socgpu_server_stats *stats);
/* Finish every queued request, then release the server. */
SOCGPU_API int socgpu_server_destroy(socgpu_server server);

/* Kernel launches made by this thread since the library loaded (profiling
 * aid, extension). */
SOCGPU_API long long socgpu_kernel_launch_count(void);

/* Select the CUDA device for this host thread (extension). */
SOCGPU_API int socgpu_set_device(int device);

/* Fix the tile shape of one kernel family (extension, used by the tuner):
 * precision SOCGPU_PRECISION_*, mode 0 = infra-red without scattering,
 * 1 = full scattering, 2 = McICA; lanes_per_solve in {8 (mixed only), 16,
 * 32} lanes sharing one (column, g-point) solve, or 1 for the phased kernel
 * (one thread per k-term for the column's recurrences; modes 0 and 1: calls
 * it does not cover -- equivalent extinction, the unscaled direct beam,
 * more than 256 layers -- run on the scan kernels); warps_per_cta in 1..8.
 * Zeros restore the built-in choice. */
SOCGPU_API int socgpu_set_tile_config(int precision, int mode, int lanes_per_solve, int warps_per_cta);

#ifdef __cplusplus
}
#endif

#endif /* SOCGPU_H */
