"""The reference's McICA test case 5118_142 (examples/netcdf/mcica/run_me) as
the Cl_run_cdf driver sets it up (src/aux/l_run_cdf.F90 with
src/aux/input_cloud_cdf.f), from the fixture made by make_mcica5118.py.

Clouds (input_cloud_cdf.f:340-400, 600-790): water and ice components of one
homogeneous cloud type (-K 1), in-cloud mixing ratios from .lwm and .iwm,
sizes from .re and .ire clamped to the range of validity of the chosen
parameter sets, the cloud fraction from .clfr.  McICA (l_run_cdf.F90:
1281-1296 and socrates_set_cld_mcica.F90): the McICA data file's counts and
tables, seeds 10 + profile, exponential overlap (i_overlap = 2) with the
decorrelation pressure scale of -dp, relative standard deviation of
condensate 0.75 (-m), optimal sampling (+m 2)."""
from dataclasses import replace
from pathlib import Path

import numpy as np

import circ6
from socrates_gb300 import abi
from socrates_gb300 import radiance as R
from socrates_gb300.spectrum import Spectrum
from socrates_gb300.synth import Column

HERE = Path(__file__).resolve().parent
FIXTURE = HERE / "mcica5118.npz"
RUNS = ("lw_avg", "sw_avg", "sw_ds0_avg", "lw_ga7", "sw_ga7")
PI = 3.14159265358979323846          # rad_ccf.F90
RAD_MCICA_SIGMA, DP_CORR_STRAT = 0.75, 10000.0
SUFFIX = {1: "q", 2: "co2", 3: "o3", 4: "n2o", 6: "ch4", 7: "o2"}


def spectra():
    """Spectra of the runs by name: GA3.0 from this fixture, GA7 from the
    CIRC case 6 fixtures."""
    return {"lw_ga3": Spectrum.load_npz(FIXTURE, prefix="lw_"), "sw_ga3": Spectrum.load_npz(FIXTURE, prefix="sw_"),
            "lw_ga7": Spectrum.load_npz(HERE / "circ6_lw_ga7.npz", prefix="sp_"),
            "sw_ga7": Spectrum.load_npz(HERE / "ga7_sw_spectrum.npz")}


def mcica_data(d, pre) -> R.McicaData:
    """The McICA data file, with the xcw columns cloud_gen reads here and NaN
    elsewhere (a read outside them would show in the results)."""
    gen, single, optimal, ipph, n1, n2, c0, c1 = (int(x) for x in d[pre + "scalars"])
    xcw = np.full((n1, n2), np.nan)
    xcw[:, c0 - 1:c1 - 1] = d[pre + "xcw_cols"]
    tab = lambda a: {(int(b), int(k)): int(n) for b, k, n in a}
    return R.McicaData(gen, single, optimal, ipph, d[pre + "reorder_single"], d[pre + "reorder_optimal"],
                       tab(d[pre + "sw_subcol_k"]), tab(d[pre + "lw_subcol_k"]), np.asfortranarray(xcw))


def setup(run, sps, precision=abi.PRECISION_FP64, n_col=1):
    """Control, spectrum, column (repeated n_col times), McICA data and the
    known-good heating rates of one run."""
    d = np.load(FIXTURE)
    solar = run.startswith("sw")
    ga7 = run.endswith("ga7")
    sp = sps[("sw_" if solar else "lw_") + ("ga7" if ga7 else "ga3")]
    f = lambda a: np.asfortranarray(np.repeat(np.asarray(a, dtype=np.float64)[None, ...], n_col, axis=0))
    p, t, p_level, t_level = f(d["p"]), f(d["t"]), f(d["p_level"]), f(d["t_level"])
    L = p.shape[1]
    gas = np.zeros((n_col, L, sp.n_absorb), order="F")
    for j, ty in enumerate(sp.type_absorb):
        if int(ty) in SUFFIX:
            gas[:, :, j] = f(d[SUFFIX[int(ty)]])
    mass = np.asfortranarray((p_level[:, 1:] - p_level[:, :-1]) / circ6.GRAV_ACC)
    q = gas[:, :, sp.index_water - 1]
    density = np.asfortranarray(p / (circ6.R_GAS_DRY * t * (1.0 + (circ6.MOL_WEIGHT_AIR / (
        circ6.MOLAR_WEIGHT_H2O * 1.0e-03) - 1.0) * q)))
    col = Column(n_col, L, p, t, p_level, t_level, mass, gas, z=np.zeros_like(p),
                 t_ground=np.full(n_col, float(d["tstar"][0])), density=density)
    col.rho_alb = np.full((n_col, 2, sp.n_band), float(d["surfsw" if solar else "surflw"][0]), order="F")
    if solar:
        col.zen_0 = np.full(n_col, 1.0 / np.cos(PI * float(d["szen"][0]) / 180.0))
        col.solar_irrad = np.full(n_col, float(d["stoa"][0]))
    # cloud components (-d, -i): the parameter-set types and their schemes
    dtype, itype = (5, 8) if ga7 else ((3, 3) if solar else (1, 1))
    scheme_w, scheme_i = int(sp.i_drop_parm[dtype - 1]), int(sp.i_ice_parm[itype - 1])
    re = np.clip(f(d["re"]), sp.drop_parm_min_dim[dtype - 1], sp.drop_parm_max_dim[dtype - 1])
    ire = np.clip(f(d["ire"]), sp.ice_parm_min_dim[itype - 1], sp.ice_parm_max_dim[itype - 1])
    w = f(d["clfr"])
    frac = np.asfortranarray(np.where(w > 0.0, 1.0, 0.0)[:, :, None])
    col.cld = dict(n_condensed=2, type_condensed=[abi.IP_PHASE_WATER, abi.IP_PHASE_ICE],
                   i_cloud_type=[1, 1], n_cloud_type=1, i_condensed_param=[scheme_w, scheme_i],
                   i_condensed_type=[dtype, itype],
                   condensed_mix_ratio=np.asfortranarray(np.stack([f(d["lwm"]), f(d["iwm"])], axis=2)),
                   condensed_dim_char=np.asfortranarray(np.stack([re, ire], axis=2)),
                   w_cloud=w, frac_cloud=frac, rel_var_dens=RAD_MCICA_SIGMA,
                   rand_seed=np.array([10 + i + 1 for i in range(n_col)], np.int32),
                   dp_corr_cloud=np.full((n_col, L), DP_CORR_STRAT, order="F"))
    common = dict(i_cloud=abi.IP_CLOUD_MCICA, l_rescale=True, i_solver=abi.IP_SOLVER_HOMOGEN_DIRECT,
                  i_scatter_method=abi.IP_SCATTER_FULL, l_flux_div=False, precision=precision,
                  i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL if ga7 else abi.IP_OVERLAP_K_EQV)
    if solar:
        ctl = R.sw_control(i_2stream=abi.IP_PIFM80 if ga7 else abi.IP_EDDINGTON, l_rayleigh=True,
                           l_continuum=False, **common)
        if run == "sw_ds0_avg":
            ctl = replace(ctl, i_direct_tau=abi.IP_DIRECT_NOSCALING)
    else:
        ctl = R.lw_control(i_2stream=abi.IP_ELSASSER, l_ir_source_quad=False, l_continuum=True, **common)
    return ctl, sp, col, mcica_data(d, "ga7_" if ga7 else "ga3_"), np.asarray(d["kgo_" + run])


def run_case(run, sps, radiance_calc, impl=None, precision=abi.PRECISION_FP64, n_col=1):
    """set_cld_mcica and radiance_calc of one run: (fluxes, McICA state,
    column, known-good heating rates)."""
    ctl, sp, col, data, kgo = setup(run, sps, precision, n_col)
    m = R.set_cld_mcica(sp, col, ctl.isolir, sampling=abi.IP_MCICA_OPTIMAL_SAMPLING, ioverlap=abi.IP_EXPONENTIAL,
                        rng=abi.RNG_LCG, data=data, impl=impl)
    return radiance_calc(ctl, sp, col, m), m, col, kgo
