"""CIRC case 6 in the short wave with the GA7 spectral file, clouds and the
overlay of prescribed soot optical properties, as the reference's Cl_run_cdf
driver sets it up (src/aux/l_run_cdf.F90, input_aerosol_cdf.f,
input_cloud_cdf.f), from the fixture made by make_circ6_sw.py.

Options (examples/netcdf/CIRC_case6/run_me: -R 1 6 -S +R -g 4 -c -r -a +A
-C 2 -K 1 -d 5 -i 8, and the Cl_run_cdf defaults): PIFM80 two-stream
coefficients, delta-rescaling with Henyey-Greenstein phase functions
(angular_control_cdf.f:236-246), the equivalent-extinction gas overlap,
continuum, Rayleigh scattering, droplet type 5 and ice type 8 of one
homogeneous cloud type in a clear and a cloudy region with maximum-random
overlap and Hogan's solver.  Aerosols: every species of the spectral file
is an entry (mr_type_index 1..26, radiatively active); none has a
mixing-ratio file, so their mixing ratios are zero, and soot (type 4)
takes the prescribed properties of case6.op_soot_hadgem in place of its
parametrization."""
from dataclasses import replace
from pathlib import Path

import numpy as np

import circ6
from socrates_gb300 import abi
from socrates_gb300 import radiance as R
from socrates_gb300.spectrum import Spectrum
from socrates_gb300.synth import Column

FIXTURE = Path(__file__).resolve().parent / "circ6_sw_ga7.npz"
PI = 3.14159265358979323846
DROP_TYPE, ICE_TYPE, SOOT = 5, 8, 4


def spectrum():
    """The GA7 short-wave spectrum with soot unparametrized (the overlay)."""
    sp = Spectrum.load_npz(FIXTURE, prefix="sp_")
    parm = np.array(sp.i_aerosol_parm, np.int32)
    parm[list(sp.type_aerosol).index(SOOT)] = abi.IP_AEROSOL_UNPARAMETRIZED
    sp.i_aerosol_parm = parm
    sp.name = "sp_sw_ga7_soot_overlay"
    return sp


def load(precision=abi.PRECISION_FP64, sp=None):
    """Control, spectrum, column and the reference's heating rates."""
    d = np.load(FIXTURE)
    sp = sp or spectrum()
    f = lambda a: np.asfortranarray(np.asarray(a, dtype=np.float64)[None, ...])
    p, t, p_level, t_level, gas = f(d["p"]), f(d["t"]), f(d["p_level"]), f(d["t_level"]), f(d["gas"])
    L = p.shape[1]
    mass = np.asfortranarray((p_level[:, 1:] - p_level[:, :-1]) / circ6.GRAV_ACC)
    q = gas[:, :, sp.index_water - 1]
    density = np.asfortranarray(p / (circ6.R_GAS_DRY * t * (1.0 + (circ6.MOL_WEIGHT_AIR / (
        circ6.MOLAR_WEIGHT_H2O * 1.0e-03) - 1.0) * q)))
    col = Column(1, L, p, t, p_level, t_level, mass, gas, z=np.zeros_like(p), t_ground=np.zeros(1),
                 density=density)
    alb = np.zeros((1, 2, sp.n_band), order="F")
    alb[0, 0, :] = d["alb"]
    alb[0, 1, :] = d["alb"]
    col.rho_alb = alb
    col.zen_0 = 1.0 / np.cos(PI * d["szen"] / 180.0)
    col.solar_irrad = np.asarray(d["stoa"], dtype=np.float64).copy()
    re = np.clip(f(d["re"]), sp.drop_parm_min_dim[DROP_TYPE - 1], sp.drop_parm_max_dim[DROP_TYPE - 1])
    ire = np.clip(f(d["ire"]), sp.ice_parm_min_dim[ICE_TYPE - 1], sp.ice_parm_max_dim[ICE_TYPE - 1])
    w = f(d["clfr"])
    col.cld = dict(n_condensed=2, type_condensed=[abi.IP_PHASE_WATER, abi.IP_PHASE_ICE], i_cloud_type=[1, 1],
                   n_cloud_type=1,
                   i_condensed_param=[int(sp.i_drop_parm[DROP_TYPE - 1]), int(sp.i_ice_parm[ICE_TYPE - 1])],
                   i_condensed_type=[DROP_TYPE, ICE_TYPE],
                   condensed_mix_ratio=np.asfortranarray(np.stack([f(d["lwm"]), f(d["iwm"])], axis=2)),
                   condensed_dim_char=np.asfortranarray(np.stack([re, ire], axis=2)),
                   w_cloud=w, frac_cloud=np.asfortranarray(np.where(w > 0.0, 1.0, 0.0)[:, :, None]))
    # aerosols: all species, zero mixing ratios, soot prescribed
    na, nb = len(sp.type_aerosol), sp.n_band
    js = list(sp.type_aerosol).index(SOOT)
    lev = np.asarray(d["soot_plev"], dtype=np.float64)
    nl, nm = lev.size, d["soot_phf"].shape[1]
    pp = np.zeros((1, nl, na), order="F")
    ab = np.zeros((1, nl, na, nb), order="F")
    sc = np.zeros((1, nl, na, nb), order="F")
    ph = np.zeros((1, nl, nm, na, nb), order="F")
    pp[0, :, js] = lev
    ab[0, :, js, :] = d["soot_abs"].T
    sc[0, :, js, :] = d["soot_scat"].T
    ph[0, :, :, js, :] = np.transpose(d["soot_phf"], (2, 1, 0))
    nlev, nmom = np.ones(na, np.int32), np.ones(na, np.int32)
    nlev[js], nmom[js] = nl, nm
    col.aer = dict(mix_ratio=np.zeros((1, L, na), order="F"), mr_type_index=np.arange(1, na + 1, dtype=np.int32),
                   mr_source=np.full(na, abi.IP_AERSRC_CLASSIC_RON, np.int32),
                   mean_rel_humidity=mean_rel_humidity(col, sp, w),
                   n_opt_level_prsc=nlev, n_phase_term_prsc=nmom, pressure_prsc=pp, absorption_prsc=ab,
                   scattering_prsc=sc, phase_fnc_prsc=ph)
    ctl = R.sw_control(i_2stream=abi.IP_PIFM80, l_rayleigh=True, l_continuum=True,
                       i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL, l_rescale=True, i_scatter_method=abi.IP_SCATTER_FULL,
                       i_cloud=abi.IP_CLOUD_MIX_MAX, i_solver=abi.IP_SOLVER_MIX_DIRECT_HOGAN, l_aerosol=True,
                       l_henyey_greenstein_pf=True, l_aerosol_mode=False, l_flux_div=False, precision=precision)
    return ctl, sp, col, np.asarray(d["kgo_hrts"])


def mean_rel_humidity(col, sp, w_cloud):
    """Clear-sky mean relative humidity of set_moist_aerosol_properties.F90
    with the saturation mixing ratio of the Goff-Gratch formula (as
    socgpu_run computes it); with zero mixing ratios it does not change the
    fluxes, it only has to lie in [0, 1)."""
    t = np.clip(col.t, 183.15, 338.15)
    r = 373.16 / t
    log10_hpa = (-7.90298 * (r - 1.0) + 5.02808 * np.log10(r) - 1.3816e-7 * (10.0 ** (11.344 * (1.0 - 1.0 / r)) - 1.0)
                 + 8.1328e-3 * (10.0 ** (-3.49149 * (r - 1.0)) - 1.0) + np.log10(1013.246))
    e = 100.0 * 10.0 ** log10_hpa * (1.0 + 1.0e-8 * col.p * (4.5 + 6.0e-4 * (col.t - 273.15) ** 2))
    eps = circ6.MOLAR_WEIGHT_H2O * 1.0e-03 / circ6.MOL_WEIGHT_AIR
    qs = eps * e / (np.maximum(col.p, e) - (1.0 - eps) * e)
    qw = col.gas_mix_ratio[:, :, sp.index_water - 1]
    clr = np.clip((qw - w_cloud * qs) / np.maximum(1.0 - w_cloud, 0.001), 0.0, qw)
    return np.asfortranarray(np.clip(clr * (1.0 - qs) / ((1.0 - clr) * qs), 0.0, 0.99999))


def heating_rate(out, col):
    return circ6.heating_rate(out, col.mass)
