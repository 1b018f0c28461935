"""The model-facing interface: set_spectrum and runes with the keyword
arguments of the reference (src/interface_core/socrates_set_spectrum.F90,
src/interface_core/socrates_runes.F90:47-200), over socgpu_runes.

    set_spectrum(spectrum_name="lw", spectral_file="sp_lw_ga9", wenyi_file=...)
    diag = runes(n_profile=1, n_layer=32, spectrum_name="lw", i_source=IP_SOURCE_THERMAL,
                 p_layer=..., t_layer=..., t_level=..., t_ground=..., mass=..., density=...,
                 h2o=..., o3=..., co2_mix_ratio=6e-4, l_grey_albedo=True, grey_albedo=0.0)

Arrays have the profile index first, as the reference's (n_profile, n_layer)
arguments.  The diagnostics come back as a dict of the StrDiag members
(heating_rate, flux_up, flux_down, flux_direct, flux_*_surf, flux_*_toa).
Clouds (set_cld, set_cld_dim, set_cld_mcica) and classic aerosol species
(set_aer) take the reference's argument names too."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .radiance import RadianceError, load_library, register_spectrum
from .spectrum import Spectrum

IP_SOURCE_ILLUMINATE, IP_SOURCE_THERMAL = abi.IP_SOURCE_ILLUMINATE, abi.IP_SOURCE_THERMAL

# runes' gas arguments by gas identifier (gas_list_pcf.F90: ip_h2o = 1 ...)
GAS_NAMES = ["h2o", "co2", "o3", "n2o", "co", "ch4", "o2", "no", "so2", "no2", "nh3", "hno3", "n2", "cfc11",
             "cfc12", "cfc113", "hcfc22", "hfc125", "hfc134a", "cfc114", "tio", "vo", "h2", "he", "ocs", "na", "k",
             "feh", "crh", "li", "rb", "cs", "ph3", "c2h2", "hcn", "h2s", "ar", None, "o", "n", "no3", "n2o5",
             "hono", "ho2no2", "h2o2", "c2h6", "ch3", "h2co", "ho2", "hdo", "hcl", "hf", "cosso", "tosso",
             "yosos", "ch3cho", "ch3ooh", "ch3coch3", "ch3cocho", "chocho", "c2h5cho", "hoch2cho", "c2h5coch3",
             "mvk", "macr", "pan", "ch3ono2"]
GAS_ID = {name: i + 1 for i, name in enumerate(GAS_NAMES) if name}

# runes' classic aerosol arguments by aerosol type (rad_pcf.F90:
# ip_water_soluble = 1 ... ip_twobindust_2 = 32; 29 is murk)
AEROSOL_NAMES = ["water_soluble", "dust_like", "oceanic", "soot", "ash", "sulphuric", "ammonium_sulphate", None,
                 "saharan_dust", "accum_sulphate", "aitken_sulphate", "fresh_soot", "aged_soot", "sodium_chloride",
                 "seasalt_film", "seasalt_jet", "dust_div1", "dust_div2", "dust_div3", "dust_div4", "dust_div5",
                 "dust_div6", "biomass_1", "biomass_2", "biogenic", "ocff_fresh", "ocff_aged", "delta", "murk",
                 "nitrate", "twobindust_1", "twobindust_2"]
AEROSOL_ID = {name: i + 1 for i, name in enumerate(AEROSOL_NAMES) if name}
CLOUD_ARRAYS = ("cloud_frac", "conv_frac", "liq_frac", "ice_frac", "liq_conv_frac", "ice_conv_frac", "liq_mmr",
                "ice_mmr", "liq_conv_mmr", "ice_conv_mmr", "liq_dim", "ice_dim", "liq_rsd", "ice_rsd",
                "liq_conv_dim", "ice_conv_dim", "liq_conv_rsd", "ice_conv_rsd")


def set_spectrum(spectrum_name: str, spectral_file=None, spectrum: Spectrum | None = None, wenyi_file=None,
                 k_file=None) -> int:
    """Read a spectral file (its '_k' tables beside it; Wen-Yi tables from
    wenyi_file, a SOCRATES source that defines them) or take a parsed
    Spectrum, and register it on the device under spectrum_name
    (socrates_set_spectrum.F90:90-121).  Returns the handle."""
    if spectrum is not None:
        spectrum.name = spectrum_name
        return register_spectrum(spectrum)
    lib = load_library()
    h = C.c_int(0)
    msg = C.create_string_buffer(512)
    enc = lambda x: None if x is None else str(x).encode()
    st = lib.socgpu_spectrum_load_ext(spectrum_name.encode(), enc(spectral_file), enc(k_file), enc(wenyi_file),
                                      C.byref(h), msg, 512)
    if st != abi.I_NORMAL:
        raise RadianceError(st, msg.value.decode())
    return h.value


def runes(n_profile: int, n_layer: int, spectrum_name: str, i_source: int, *, p_layer, t_layer, mass,
          density=None, p_level=None, t_level=None, t_ground=None, l_flux_ground=False, flux_ground=None,
          cos_zenith_angle=None, solar_irrad=None, l_grey_albedo=False, grey_albedo=0.0, albedo_diff=None,
          albedo_dir=None, l_tile=False, n_tile=0, l_flux_tile=None, frac_tile=None, t_tile=None, flux_tile=None,
          albedo_diff_tile=None, albedo_dir_tile=None, i_scatter_method=0, i_gas_overlap=0, l_rayleigh=False,
          l_mixing_ratio=False, l_aerosol_mode=False, n_aer_mode=0, aer_mix_ratio=None, aer_absorption=None,
          aer_scattering=None, aer_asymmetry=None, layer_heat_capacity=None, l_invert=False,
          precision=abi.PRECISION_FP64, mean_rel_humidity=None, i_cloud_representation=0, i_overlap=0,
          i_inhom=0, i_cloud_entrapment=0, i_mcica_sampling=-1, i_st_water=0, i_st_ice=0, i_drop_re=0,
          n_cloud_layer=0, liq_dim_constant=None, cloud_vertical_decorr=None, cloud_horizontal_rsd=None,
          rand_seed=None, mcica_data=None, i_cnv_water=0, i_cnv_ice=0, liq_conv_dim_constant=None,
          conv_vertical_decorr=None, **kw) -> dict:
    """runes (socrates_runes.F90:47) through socgpu_runes.  Gases are passed
    by the reference's names: <gas> a profile (n_profile, n_layer),
    <gas>_mix_ratio a well-mixed value, l_<gas>_well_mixed to prefer it.
    Classic aerosols by the names of set_aer (water_soluble, dust_like, ...
    each a (n_profile, n_layer) mixing ratio; l_<name>=False drops one).
    Clouds by the names of set_cld and set_cld_dim (cloud_frac, liq_mmr,
    liq_dim, ...); mcica_data is the path of the McICA data file."""
    lib = load_library()
    keep = []

    def dp(x, dtype=np.float64):
        if x is None:
            return None
        a = np.asfortranarray(np.asarray(x, dtype=dtype))
        keep.append(a)
        return a.ctypes.data_as(C.POINTER(C.c_double if dtype == np.float64 else C.c_int))

    a = abi.RunesArgs()
    a.n_profile, a.n_layer, a.i_source = n_profile, n_layer, i_source
    name = spectrum_name.encode()
    a.spectrum_name = name
    a.p_layer, a.t_layer, a.mass, a.density = dp(p_layer), dp(t_layer), dp(mass), dp(density)
    a.p_level, a.t_level = dp(p_level), dp(t_level)
    aer_flags = {k[2:]: bool(v) for k, v in kw.items() if k.startswith("l_") and k[2:] in AEROSOL_ID}
    gases = {}
    for key, val in kw.items():
        if key.startswith("l_") and key[2:] in AEROSOL_ID:
            continue
        if key in AEROSOL_ID:
            if aer_flags.get(key, True) and val is not None:
                a.aerosol[AEROSOL_ID[key]] = dp(val)
        elif key in CLOUD_ARRAYS:
            setattr(a, key, dp(val))
        else:
            gases[key] = val
    a.mean_rel_humidity = dp(mean_rel_humidity)
    a.i_cloud_representation, a.i_overlap, a.i_inhom = int(i_cloud_representation), int(i_overlap), int(i_inhom)
    a.i_cloud_entrapment, a.i_mcica_sampling = int(i_cloud_entrapment), int(i_mcica_sampling)
    a.i_st_water, a.i_st_ice, a.i_drop_re, a.n_cloud_layer = int(i_st_water), int(i_st_ice), int(i_drop_re), \
        int(n_cloud_layer)
    a.i_cnv_water, a.i_cnv_ice = int(i_cnv_water), int(i_cnv_ice)
    for name, val in (("liq_dim_constant", liq_dim_constant), ("cloud_vertical_decorr", cloud_vertical_decorr),
                      ("cloud_horizontal_rsd", cloud_horizontal_rsd), ("liq_conv_dim_constant", liq_conv_dim_constant),
                      ("conv_vertical_decorr", conv_vertical_decorr)):
        if val is not None:
            setattr(a, name, float(val))
            setattr(a, "has_" + name, 1)
    if rand_seed is not None:
        a.rand_seed = dp(np.asarray(rand_seed, dtype=np.int32), np.int32)
    mcica_path = None if mcica_data is None else str(mcica_data).encode()
    a.mcica_data = mcica_path
    for key, val in gases.items():
        if key.startswith("l_") and key.endswith("_well_mixed"):
            gid = GAS_ID.get(key[2:-len("_well_mixed")])
            if gid is None:
                raise TypeError(f"runes() got an unexpected keyword argument '{key}'")
            a.gas_well_mixed[gid] = int(bool(val))
        elif key.endswith("_mix_ratio"):
            gid = GAS_ID.get(key[:-len("_mix_ratio")])
            if gid is None:
                raise TypeError(f"runes() got an unexpected keyword argument '{key}'")
            a.gas_mix_ratio[gid] = float(val)
            a.has_mix_ratio[gid] = 1
        elif key in GAS_ID:
            a.gas[GAS_ID[key]] = dp(val)
        else:
            raise TypeError(f"runes() got an unexpected keyword argument '{key}'")
    a.l_invert = int(l_invert)
    a.t_ground = dp(t_ground)
    a.l_flux_ground, a.flux_ground = int(l_flux_ground), dp(flux_ground)
    a.cos_zenith_angle, a.solar_irrad = dp(cos_zenith_angle), dp(solar_irrad)
    a.l_grey_albedo, a.grey_albedo = int(l_grey_albedo), float(grey_albedo)
    a.albedo_diff, a.albedo_dir = dp(albedo_diff), dp(albedo_dir)
    a.l_tile, a.n_tile = int(l_tile), int(n_tile)
    a.l_flux_tile = dp(None if l_flux_tile is None else np.asarray(l_flux_tile, dtype=np.int32), np.int32)
    a.frac_tile, a.t_tile, a.flux_tile = dp(frac_tile), dp(t_tile), dp(flux_tile)
    a.albedo_diff_tile, a.albedo_dir_tile = dp(albedo_diff_tile), dp(albedo_dir_tile)
    a.i_scatter_method, a.i_gas_overlap = int(i_scatter_method), int(i_gas_overlap)
    a.l_rayleigh, a.l_mixing_ratio = int(l_rayleigh), int(l_mixing_ratio)
    a.l_aerosol_mode, a.n_aer_mode = int(l_aerosol_mode), int(n_aer_mode)
    a.aer_mix_ratio, a.aer_absorption = dp(aer_mix_ratio), dp(aer_absorption)
    a.aer_scattering, a.aer_asymmetry = dp(aer_scattering), dp(aer_asymmetry)
    a.layer_heat_capacity = dp(layer_heat_capacity)
    a.precision = int(precision)
    out = {k: np.zeros((n_profile, n_layer + 1), order="F") for k in ("flux_up", "flux_down", "flux_direct")}
    out["heating_rate"] = np.zeros((n_profile, n_layer), order="F")
    for k in ("flux_up_surf", "flux_down_surf", "flux_direct_surf", "flux_up_toa", "flux_down_toa",
              "flux_direct_toa"):
        out[k] = np.zeros(n_profile)
    d = abi.RunesDiag()
    for k, v in out.items():
        setattr(d, k, v.ctypes.data_as(C.POINTER(C.c_double)))
    msg = C.create_string_buffer(512)
    st = lib.socgpu_runes(C.byref(a), C.byref(d), msg, 512)
    if st != abi.I_NORMAL:
        raise RadianceError(st, msg.value.decode())
    return out
