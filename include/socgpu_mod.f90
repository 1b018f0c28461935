! socgpu_mod.f90 -- iso_c_binding interface of libsocgpu for Fortran hosts.
!
! The derived types mirror the C structs of socgpu.h member by member (the
! CPU test tests/test_fortran_module.py checks names, kinds and order
! against the C layouts); the interfaces bind the entry points a model that
! calls radiance_calc (src/radiance_core/radiance_calc.F90:16) or runes
! (src/interface_core/socrates_runes.F90:47) uses instead.  A caller fills
! the C views with c_loc of its contiguous arrays, LOGICALs as 0 or 1, and
! absent optional arrays as C_NULL_PTR (INTEGRATION.md shows the call sites).
MODULE socgpu_mod
USE, INTRINSIC :: iso_c_binding
IMPLICIT NONE

TYPE, BIND(C) :: socgpu_control
  INTEGER(c_int) :: isolir, i_angular_integration, i_2stream, i_scatter_method, &
                    i_solver, i_cloud, i_cloud_representation, i_gas_overlap,  &
                    i_direct_tau, l_rescale, n_order_forward, l_ir_source_quad,&
                    l_rayleigh, l_gas, l_aerosol_mode, l_flux_div,             &
                    first_band, last_band
  TYPE(c_ptr)    :: weight_band
  INTEGER(c_int) :: precision, l_continuum, l_mixing_ratio, l_grey_single
  INTEGER(c_int) :: l_aerosol, l_henyey_greenstein_pf
END TYPE

TYPE, BIND(C) :: socgpu_dimen
  INTEGER(c_int) :: nd_profile, nd_layer, id_cloud_top, nd_aerosol_mode, &
                    nd_cloud_component, nd_cloud_type, nd_subcol_gen, nd_subcol_req, &
                    nd_aerosol_mr, nd_profile_aerosol_prsc, nd_opt_level_aerosol_prsc, &
                    nd_phf_term_aerosol_prsc
END TYPE

TYPE, BIND(C) :: socgpu_atm
  INTEGER(c_int) :: n_profile, n_layer
  TYPE(c_ptr)    :: p, t, p_level, t_level, mass, gas_mix_ratio, density
END TYPE

TYPE, BIND(C) :: socgpu_bound
  TYPE(c_ptr) :: zen_0, solar_irrad, rho_alb, t_ground, flux_ground
END TYPE

TYPE, BIND(C) :: socgpu_aer
  INTEGER(c_int) :: n_mode
  TYPE(c_ptr)    :: mode_mix_ratio, mode_absorption, mode_scattering, mode_asymmetry
  INTEGER(c_int) :: n_aerosol_mr
  TYPE(c_ptr)    :: mix_ratio, mr_type_index, mr_source, mean_rel_humidity
  TYPE(c_ptr)    :: n_opt_level_prsc, n_phase_term_prsc, pressure_prsc, absorption_prsc, &
                    scattering_prsc, phase_fnc_prsc
END TYPE

TYPE, BIND(C) :: socgpu_cld
  INTEGER(c_int) :: n_condensed
  TYPE(c_ptr)    :: type_condensed, i_cloud_type, i_condensed_param, i_condensed_type, &
                    condensed_mix_ratio, condensed_dim_char
  INTEGER(c_int) :: n_cloud_type
  TYPE(c_ptr)    :: w_cloud, frac_cloud
  INTEGER(c_int) :: n_subcol_gen, n_subcol_req
  TYPE(c_ptr)    :: c_sub, frac_cloudy, n_subcol_cld, subcol_k, first_subcol_k, subcol_reorder
  REAL(c_double) :: dp_corr_strat, dp_corr_conv
END TYPE

TYPE, BIND(C) :: socgpu_radout
  TYPE(c_ptr) :: flux_up, flux_down, flux_direct, flux_div, heating_rate, &
                 flux_up_band, flux_down_band
END TYPE

INTEGER, PARAMETER :: socgpu_runes_n_gas = 80
INTEGER, PARAMETER :: socgpu_runes_n_aer = 33

TYPE, BIND(C) :: socgpu_runes_args
  INTEGER(c_int) :: n_profile, n_layer
  TYPE(c_ptr)    :: spectrum_name
  INTEGER(c_int) :: i_source
  TYPE(c_ptr)    :: p_layer, t_layer, mass, density, p_level, t_level
  TYPE(c_ptr)    :: gas(socgpu_runes_n_gas)
  REAL(c_double) :: gas_mix_ratio(socgpu_runes_n_gas)
  INTEGER(c_int) :: has_mix_ratio(socgpu_runes_n_gas), gas_well_mixed(socgpu_runes_n_gas)
  INTEGER(c_int) :: l_invert
  TYPE(c_ptr)    :: t_ground
  INTEGER(c_int) :: l_flux_ground
  TYPE(c_ptr)    :: flux_ground, cos_zenith_angle, solar_irrad
  INTEGER(c_int) :: l_grey_albedo
  REAL(c_double) :: grey_albedo
  TYPE(c_ptr)    :: albedo_diff, albedo_dir
  INTEGER(c_int) :: l_tile, n_tile
  TYPE(c_ptr)    :: l_flux_tile, frac_tile, t_tile, flux_tile, albedo_diff_tile, albedo_dir_tile
  INTEGER(c_int) :: i_scatter_method, i_gas_overlap, l_rayleigh, l_mixing_ratio
  INTEGER(c_int) :: l_aerosol_mode, n_aer_mode
  TYPE(c_ptr)    :: aer_mix_ratio, aer_absorption, aer_scattering, aer_asymmetry
  TYPE(c_ptr)    :: layer_heat_capacity
  INTEGER(c_int) :: precision
  TYPE(c_ptr)    :: aerosol(socgpu_runes_n_aer)
  TYPE(c_ptr)    :: mean_rel_humidity
  INTEGER(c_int) :: i_cloud_representation, i_overlap, i_inhom, i_cloud_entrapment, &
                    i_mcica_sampling, i_st_water, i_st_ice, i_drop_re, n_cloud_layer
  TYPE(c_ptr)    :: cloud_frac, conv_frac, liq_frac, ice_frac, liq_conv_frac, ice_conv_frac, &
                    liq_mmr, ice_mmr, liq_conv_mmr, ice_conv_mmr, liq_dim, ice_dim, liq_rsd, ice_rsd
  INTEGER(c_int) :: has_liq_dim_constant, has_cloud_vertical_decorr, has_cloud_horizontal_rsd
  REAL(c_double) :: liq_dim_constant, cloud_vertical_decorr, cloud_horizontal_rsd
  TYPE(c_ptr)    :: rand_seed, mcica_data
  INTEGER(c_int) :: i_cnv_water, i_cnv_ice
  TYPE(c_ptr)    :: liq_conv_dim, ice_conv_dim, liq_conv_rsd, ice_conv_rsd
  INTEGER(c_int) :: has_liq_conv_dim_constant
  REAL(c_double) :: liq_conv_dim_constant
  INTEGER(c_int) :: has_conv_vertical_decorr
  REAL(c_double) :: conv_vertical_decorr
END TYPE

TYPE, BIND(C) :: socgpu_runes_diag
  TYPE(c_ptr) :: heating_rate, flux_up, flux_down, flux_direct,     &
                 flux_up_surf, flux_down_surf, flux_direct_surf,    &
                 flux_up_toa, flux_down_toa, flux_direct_toa
END TYPE

INTERFACE
  INTEGER(c_int) FUNCTION socgpu_radiance_calc(control, dimen, spectrum, atm, cld, aer, &
      bound, radout, msg, msg_len) BIND(C, NAME='socgpu_radiance_calc')
    IMPORT
    TYPE(socgpu_control), INTENT(IN)    :: control
    TYPE(socgpu_dimen),   INTENT(IN)    :: dimen
    INTEGER(c_int32_t),   VALUE         :: spectrum
    TYPE(socgpu_atm),     INTENT(IN)    :: atm
    TYPE(socgpu_cld),     INTENT(IN)    :: cld
    TYPE(socgpu_aer),     INTENT(IN)    :: aer
    TYPE(socgpu_bound),   INTENT(IN)    :: bound
    TYPE(socgpu_radout),  INTENT(IN)    :: radout
    CHARACTER(KIND=c_char), INTENT(OUT) :: msg(*)
    INTEGER(c_size_t),    VALUE         :: msg_len
  END FUNCTION

  INTEGER(c_int) FUNCTION socgpu_runes(args, diag, msg, msg_len) BIND(C, NAME='socgpu_runes')
    IMPORT
    TYPE(socgpu_runes_args), INTENT(IN) :: args
    TYPE(socgpu_runes_diag), INTENT(IN) :: diag
    CHARACTER(KIND=c_char), INTENT(OUT) :: msg(*)
    INTEGER(c_size_t), VALUE            :: msg_len
  END FUNCTION

  INTEGER(c_int) FUNCTION socgpu_spectrum_load_ext(name, path, k_path, wenyi_path, handle, &
      msg, msg_len) BIND(C, NAME='socgpu_spectrum_load_ext')
    IMPORT
    CHARACTER(KIND=c_char), INTENT(IN) :: name(*), path(*)
    TYPE(c_ptr), VALUE                 :: k_path, wenyi_path    ! C_NULL_PTR: defaults
    INTEGER(c_int32_t), INTENT(OUT)    :: handle
    CHARACTER(KIND=c_char), INTENT(OUT) :: msg(*)
    INTEGER(c_size_t), VALUE           :: msg_len
  END FUNCTION

  INTEGER(c_int) FUNCTION socgpu_spectrum_lookup(name, handle) &
      BIND(C, NAME='socgpu_spectrum_lookup')
    IMPORT
    CHARACTER(KIND=c_char), INTENT(IN) :: name(*)
    INTEGER(c_int32_t), INTENT(OUT)    :: handle
  END FUNCTION

  INTEGER(c_int) FUNCTION socgpu_cloud_gen(nd_layer, cloud_top, n_layer, nd_profile, il1, il2, &
      n_subcol, n1, n2, ipph, ioverlap, rand_seed, rlc_cf, rlc_cw, sigma_qcw, avg_cf,    &
      c_cloud, c_ratio, zf, xcw, n_subcol_cld, c_sub, rng, msg, msg_len)                 &
      BIND(C, NAME='socgpu_cloud_gen')
    IMPORT
    INTEGER(c_int), VALUE :: nd_layer, cloud_top, n_layer, nd_profile, il1, il2, n_subcol, &
                             n1, n2, ipph, ioverlap, rng
    INTEGER(c_int), INTENT(IN)  :: rand_seed(*)
    REAL(c_double), INTENT(IN)  :: rlc_cf(*), rlc_cw(*), sigma_qcw(*), avg_cf(*), &
                                   c_cloud(*), c_ratio(*), zf(*), xcw(*)
    INTEGER(c_int), INTENT(OUT) :: n_subcol_cld(*)
    REAL(c_double), INTENT(OUT) :: c_sub(*)
    CHARACTER(KIND=c_char), INTENT(OUT) :: msg(*)
    INTEGER(c_size_t), VALUE    :: msg_len
  END FUNCTION

  INTEGER(c_int) FUNCTION socgpu_abi_version() BIND(C, NAME='socgpu_abi_version')
    IMPORT
  END FUNCTION

  INTEGER(c_int) FUNCTION socgpu_spectrum_load(name, path, handle, msg, msg_len) &
      BIND(C, NAME='socgpu_spectrum_load')
    IMPORT
    CHARACTER(KIND=c_char), INTENT(IN) :: name(*), path(*)
    INTEGER(c_int32_t), INTENT(OUT)    :: handle
    CHARACTER(KIND=c_char), INTENT(OUT) :: msg(*)
    INTEGER(c_size_t), VALUE           :: msg_len
  END FUNCTION

  INTEGER(c_int) FUNCTION socgpu_spectrum_n_gpoint(handle) BIND(C, NAME='socgpu_spectrum_n_gpoint')
    IMPORT
    INTEGER(c_int32_t), VALUE :: handle
  END FUNCTION

  INTEGER(c_int) FUNCTION socgpu_spectrum_release(handle) BIND(C, NAME='socgpu_spectrum_release')
    IMPORT
    INTEGER(c_int32_t), VALUE :: handle
  END FUNCTION
END INTERFACE
END MODULE socgpu_mod
