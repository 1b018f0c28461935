"""The reference's runes test (examples/runes, src/aux/runes_driver.f90) from
the fixture made by make_runes_ga9.py: the driver's arguments for each of
its four calls, and the same calls set up directly for radiance_calc with
the defaults runes gives (socrates_set_control.F90:232-300), so that the
oracle can be checked against the known-good output and socgpu_runes against
the oracle."""
from pathlib import Path

import numpy as np

from socrates_gb300 import abi
from socrates_gb300 import radiance as R
from socrates_gb300.spectrum import Spectrum
from socrates_gb300.synth import Column

FIXTURE = Path(__file__).resolve().parent / "runes_ga9.npz"
SECTIONS = ("sw", "lw_tground", "lw_flux_ground", "lw_tiles")
SECONDS_PER_DAY = 8.64e+04


def data():
    return np.load(FIXTURE)


def spectra():
    return (Spectrum.load_npz(FIXTURE, prefix="sw_"), Spectrum.load_npz(FIXTURE, prefix="lw_"))


def derived(d):
    """The driver's layer mass, density and heat capacity
    (runes_driver.f90: d_mass, density, layer_heat_capacity)."""
    p_level, p_layer, t_layer = d["p_level"], d["p_layer"], d["t_layer"]
    mass = (p_level[1:] - p_level[:-1]) / d["grav_acc"]
    density = p_layer / (d["r_gas_dry"] * t_layer)
    return mass, density, mass * d["cp_air_dry"]


def runes_kwargs(d, section):
    """The keyword arguments of the driver's runes call for one section."""
    mass, density, lhc = derived(d)
    f = lambda a: np.asfortranarray(np.asarray(a, dtype=np.float64)[None, :])
    kw = dict(n_profile=1, n_layer=32, p_layer=f(d["p_layer"]), t_layer=f(d["t_layer"]), mass=f(mass),
              density=f(density), layer_heat_capacity=f(lhc), h2o=f(d["h2o"]), o3=f(d["o3"]),
              co2_mix_ratio=float(d["co2_mix_ratio"]), n2o_mix_ratio=float(d["n2o_mix_ratio"]),
              ch4_mix_ratio=float(d["ch4_mix_ratio"]), l_grey_albedo=True, l_invert=False)
    if section == "sw":
        kw.update(spectrum_name="sw", i_source=abi.IP_SOURCE_ILLUMINATE, o2_mix_ratio=float(d["o2_mix_ratio"]),
                  cos_zenith_angle=np.array(d["cos_zenith_angle"]), solar_irrad=np.array([float(d["solar_irrad"])]),
                  grey_albedo=float(d["grey_albedo_sw"]), l_rayleigh=True)
        return kw
    kw.update(spectrum_name="lw", i_source=abi.IP_SOURCE_THERMAL, t_level=f(d["t_level"]),
              grey_albedo=float(d["grey_albedo_lw"]))
    if section == "lw_tground":
        kw.update(t_ground=np.array([float(d["t_ground"])]))
    elif section == "lw_flux_ground":
        kw.update(l_flux_ground=True, flux_ground=np.asfortranarray(d["flux_ground"].reshape(1, -1)))
    else:
        kw.update(l_tile=True, n_tile=2, l_flux_tile=d["l_flux_tile"],
                  flux_tile=np.asfortranarray(d["flux_tile"].reshape(1, 2, -1, order="F")),
                  t_tile=np.full((1, 2), float(d["t_tile"])), frac_tile=np.asfortranarray(d["frac_tile"].reshape(1, 2)))
    return kw


def planck_band(sp, b, t):
    """planck_flux_band (planck_flux_band_mod.F90:33-48)."""
    c = sp.thermal_coeff[:, b]
    x = t / sp.t_ref_planck
    v = c[sp.n_deg_fit]
    for j in range(sp.n_deg_fit - 1, -1, -1):
        v = v * x + c[j]
    return v


def direct_case(d, sw, lw, section):
    """The same call for radiance_calc: control with runes' defaults, column,
    and the surface Planck flux per band where the call gives it."""
    mass, density, _ = derived(d)
    f = lambda a: np.asfortranarray(np.asarray(a, dtype=np.float64)[None, :])
    solar = section == "sw"
    sp = sw if solar else lw
    species = {1: d["h2o"], 3: d["o3"], 2: float(d["co2_mix_ratio"]), 4: float(d["n2o_mix_ratio"]),
               6: float(d["ch4_mix_ratio"])}
    if solar:
        species[7] = float(d["o2_mix_ratio"])
    gas = np.zeros((1, 32, sp.n_absorb), order="F")
    for j, ty in enumerate(sp.type_absorb):
        v = species.get(int(ty))
        if v is not None:
            gas[0, :, j] = np.maximum(v, 0.0) if np.ndim(v) else v
    t_level = f(d["t_level"]) if not solar else np.zeros((1, 33), order="F")
    col = Column(1, 32, f(d["p_layer"]), f(d["t_layer"]), f(d["p_level"]), t_level, f(mass), gas,
                 z=np.zeros((1, 32)), t_ground=np.array([float(d["t_ground"])]), density=f(density))
    alb = float(d["grey_albedo_sw"] if solar else d["grey_albedo_lw"])
    col.rho_alb = np.full((1, 2, sp.n_band), alb, order="F")
    if solar:
        col.zen_0 = 1.0 / np.array(d["cos_zenith_angle"])
        col.solar_irrad = np.array([float(d["solar_irrad"])])
        ctl = R.sw_control(l_rayleigh=True, l_continuum=True, l_rescale=True, l_flux_div=False,
                           i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL)
    else:
        ctl = R.lw_control(l_continuum=True, l_rescale=True, l_ir_source_quad=True, l_flux_div=False,
                           i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL)
        if section == "lw_flux_ground":
            col.flux_ground = np.asfortranarray((d["flux_ground"] / (1.0 - alb)).reshape(1, -1))
        elif section == "lw_tiles":
            frac, ft, lf = d["frac_tile"], d["flux_tile"].reshape(2, -1, order="F"), d["l_flux_tile"]
            fg = np.zeros(sp.n_band)
            for b in range(sp.n_band):
                for k in range(2):
                    tile = ft[k, b] / (1.0 - alb) if lf[k] else planck_band(sp, b, float(d["t_tile"]))
                    fg[b] = frac[k] * tile if k == 0 else fg[b] + frac[k] * tile
            col.flux_ground = fg.reshape(1, -1)
    return ctl, sp, col


def printed(out, lhc):
    """The driver's printed columns for levels 1..32: flux down, flux up and
    heating rate in K/day (socrates_set_diag.F90:150-170 with the layer heat
    capacity)."""
    fd, fu = out["flux_down"][0], out["flux_up"][0]
    div = fd[:-1] - fd[1:] + fu[1:] - fu[:-1]
    return np.stack([fd[1:], fu[1:], div / lhc * SECONDS_PER_DAY], axis=1)
