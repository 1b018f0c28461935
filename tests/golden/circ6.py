"""CIRC case 6, clear-sky long wave with the GA7 spectral file, as the
reference's Cl_run_cdf driver sets it up (src/aux/l_run_cdf.F90), from the
fixture made by make_circ6.py.

Options (examples/netcdf/CIRC_case6/run_me and the Cl_run_cdf defaults,
sbin/Cl_run_cdf:278-310): infra-red, bands 1-9, gas absorption with the
equivalent-extinction overlap (-g 4), water-vapour continuum, Elsasser
two-stream (12), no rescaling, full scattering treatment, solver 13 (homogen
direct), linear IR source, clear sky.  Layer mass from the level pressures and
moist density as in l_run_cdf.F90:1205-1235; heating rates from the net
fluxes as in l_run_cdf.F90:1340-1375."""
from pathlib import Path

import numpy as np

from socrates_gb300 import abi
from socrates_gb300 import radiance as R
from socrates_gb300.spectrum import Spectrum
from socrates_gb300.synth import Column

FIXTURE = Path(__file__).resolve().parent / "circ6_lw_ga7.npz"
# rad_ccf.F90:42-58, gas_list_pcf.F90:303-306
GRAV_ACC, R_GAS_DRY, MOL_WEIGHT_AIR, CP_AIR_DRY = 9.80665, 287.026, 28.966e-03, 1.005e+03
MOLAR_WEIGHT_H2O = 18.0153


def load(precision=abi.PRECISION_FP64, n_col=1):
    """Control, spectrum, column (repeated n_col times) and the reference's
    heating rates."""
    d = np.load(FIXTURE)
    sp = Spectrum.load_npz(FIXTURE, prefix="sp_")
    f = lambda a: np.asfortranarray(np.repeat(np.asarray(a, dtype=np.float64)[None, ...], n_col, axis=0))
    p, t = f(d["p"]), f(d["t"])
    p_level, t_level = f(d["p_level"]), f(d["t_level"])
    gas = f(d["gas"])
    n_layer = p.shape[1]
    mass = np.asfortranarray((p_level[:, 1:] - p_level[:, :-1]) / GRAV_ACC)
    q = gas[:, :, sp.index_water - 1]
    density = np.asfortranarray(p / (R_GAS_DRY * t * (1.0 + (MOL_WEIGHT_AIR / (MOLAR_WEIGHT_H2O * 1.0e-03) - 1.0)
                                                       * q)))
    col = Column(n_col, n_layer, p, t, p_level, t_level, mass, gas, z=np.zeros_like(p),
                 t_ground=np.full(n_col, float(d["t_ground"][0])), density=density)
    alb = np.zeros((n_col, 2, sp.n_band), order="F")
    alb[:, :, :] = float(d["alb"][0])
    col.rho_alb = alb
    ctl = R.lw_control(i_2stream=abi.IP_ELSASSER, i_scatter_method=abi.IP_SCATTER_FULL,
                       i_solver=abi.IP_SOLVER_HOMOGEN_DIRECT, l_rescale=False, l_ir_source_quad=False,
                       l_continuum=True, l_flux_div=False, i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL,
                       precision=precision)
    return ctl, sp, col, np.asarray(d["kgo_hrts"])


def heating_rate(out, mass):
    """l_run_cdf.F90:1340-1375."""
    net = out["flux_down"] - out["flux_up"]
    return 8.64e+04 * (net[:, :-1] - net[:, 1:]) / (mass * CP_AIR_DRY)
