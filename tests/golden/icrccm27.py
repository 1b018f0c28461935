"""ICRCCM case 27 as the reference's Cl_run_cdl driver sets it up
(src/aux/l_run_cdl.F90), from the fixture made by make_icrccm27.py.

Options (examples/aer_cmp/run27 and the Cl_run_cdl defaults,
sbin/Cl_run_cdl): infra-red, bands 1-8, gas absorption with random overlap,
water-vapour continuum, Elsasser two-stream (12), no rescaling, full
scattering treatment, solver 13 (homogen direct), linear IR source, clear
sky.  Layer mass from the level pressures and moist density as in
l_run_cdl.F90:1017-1045; heating rates from the net fluxes as in
l_run_cdl.F90:1105-1124."""
from pathlib import Path

import numpy as np

from socrates_gb300 import abi
from socrates_gb300 import radiance as R
from socrates_gb300.spectrum import Spectrum
from socrates_gb300.synth import Column

FIXTURE = Path(__file__).resolve().parent / "icrccm27_lw_hadcm3.npz"
# rad_ccf.F90:42-58, gas_list_pcf.F90:303-306
GRAV_ACC, R_GAS_DRY, MOL_WEIGHT_AIR, CP_AIR_DRY = 9.80665, 287.026, 28.966e-03, 1.005e+03
MOLAR_WEIGHT_H2O = 18.0153


def load(precision=abi.PRECISION_FP64):
    d = np.load(FIXTURE)
    sp = Spectrum.load_npz(FIXTURE, prefix="sp_")
    f = lambda a: np.asfortranarray(np.asarray(a, dtype=np.float64)[None, ...])
    p, t = f(d["p"]), f(d["t"])
    p_level, t_level = f(d["p_level"]), f(d["t_level"])
    gas = np.asfortranarray(d["gas"][None, :, :])
    n_layer = p.shape[1]
    mass = np.asfortranarray((p_level[:, 1:] - p_level[:, :-1]) / GRAV_ACC)
    q = gas[:, :, sp.index_water - 1]
    density = np.asfortranarray(p / (R_GAS_DRY * t * (1.0 + (MOL_WEIGHT_AIR / (MOLAR_WEIGHT_H2O * 1.0e-03) - 1.0)
                                                       * q)))
    col = Column(1, n_layer, p, t, p_level, t_level, mass, gas, z=np.zeros_like(p),
                 t_ground=np.asarray(d["t_ground"], dtype=np.float64).reshape(1), density=density)
    alb = np.zeros((1, 2, sp.n_band), order="F")
    alb[:, :, :] = float(d["alb"][0])
    col.rho_alb = alb
    ctl = R.lw_control(i_2stream=abi.IP_ELSASSER, i_scatter_method=abi.IP_SCATTER_FULL,
                       i_solver=abi.IP_SOLVER_HOMOGEN_DIRECT, l_rescale=False, l_ir_source_quad=False,
                       l_continuum=True, l_flux_div=False, precision=precision)
    return ctl, sp, col, np.asarray(d["kgo_hrts"])


def heating_rate(out, mass):
    """l_run_cdl.F90:1105-1124."""
    net = out["flux_down"] - out["flux_up"]
    return 8.64e+04 * (net[:, :-1] - net[:, 1:]) / (mass * CP_AIR_DRY)
