"""The reference's cloud-region test case 7460_28 (examples/netcdf/7460_28/
run_me) as the Cl_run_cdf driver sets it up (src/aux/l_run_cdf.F90,
src/aux/input_cloud_cdf.f, src/aux/assign_surface_char_cdf.f), from the
fixture made by make_cld7460.py.

Clouds: water and ice of one homogeneous type (-K 1) in a clear and a cloudy
region with maximum-random overlap (-C 2); in-cloud mixing ratios from .lwm
and .iwm, sizes from .re and .ire clamped to the range of the chosen
parameter sets, fractions from .clfr.  Surfaces: one albedo weight (diffuse
and direct alike) or two (.surfsw2: diffuse, direct;
assign_surface_char_cdf.f:300-350)."""
from dataclasses import replace
from pathlib import Path

import numpy as np

import circ6
from socrates_gb300 import abi
from socrates_gb300 import radiance as R
from socrates_gb300.spectrum import Spectrum
from socrates_gb300.synth import Column

HERE = Path(__file__).resolve().parent
FIXTURE = HERE / "cld7460.npz"
RUNS = ("lw_avg", "sw_avg", "sw_ds0_avg", "sw2", "sw2_ds0", "sw_ga9_avg", "lw_ga9_avg", "ipa_lw", "ipa_sw")
PI = 3.14159265358979323846
SUFFIX = {1: "q", 2: "co2", 3: "o3", 4: "n2o", 6: "ch4", 7: "o2"}


def spectra():
    ga9 = HERE / "runes_ga9.npz"
    return {"hlw": Spectrum.load_npz(FIXTURE, prefix="hlw_"), "hsw": Spectrum.load_npz(FIXTURE, prefix="hsw_"),
            "ga9lw": Spectrum.load_npz(ga9, prefix="lw_"), "ga9sw": Spectrum.load_npz(ga9, prefix="sw_")}


def setup(run, sps, precision=abi.PRECISION_FP64):
    """Control, spectrum, column, the known-good values and their kind
    ("hrts": heating rates of the layers, "nflx": net flux of the levels)."""
    d = np.load(FIXTURE)
    solar = "sw" in run
    ga9 = "ga9" in run
    pre = "ipa_" if run.startswith("ipa") else "avg_"
    sp = sps[("ga9" if ga9 else "h") + ("sw" if solar else "lw")]
    n = d[pre + "t"].shape[1]
    f = lambda a: np.asfortranarray(np.asarray(a, dtype=np.float64).T)          # (levels, columns) -> (columns, levels)
    bc = lambda a: np.asfortranarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (n, len(a))))
    p, p_level = bc(d[pre + "p"]), bc(d[pre + "p_level"])
    t, t_level = f(d[pre + "t"]), f(d[pre + "t_level"])
    L = p.shape[1]
    gas = np.zeros((n, L, sp.n_absorb), order="F")
    for j, ty in enumerate(sp.type_absorb):
        if int(ty) in SUFFIX:
            gas[:, :, j] = f(d[pre + SUFFIX[int(ty)]])
    mass = np.asfortranarray((p_level[:, 1:] - p_level[:, :-1]) / circ6.GRAV_ACC)
    q = gas[:, :, sp.index_water - 1]
    density = np.asfortranarray(p / (circ6.R_GAS_DRY * t * (1.0 + (circ6.MOL_WEIGHT_AIR / (
        circ6.MOLAR_WEIGHT_H2O * 1.0e-03) - 1.0) * q)))
    col = Column(n, L, p, t, p_level, t_level, mass, gas, z=np.zeros_like(p), t_ground=d[pre + "tstar"].copy(),
                 density=density)
    alb = np.zeros((n, 2, sp.n_band), order="F")
    if run.startswith("sw2") or ga9 and solar:
        alb[:, 0, :], alb[:, 1, :] = d["avg_surfsw2"][0], d["avg_surfsw2"][1]
    else:
        a = d[pre + ("surfsw" if solar else "surflw")]
        alb[:, 0, :] = a[:, None]
        alb[:, 1, :] = a[:, None]
    col.rho_alb = alb
    if solar:
        col.zen_0 = 1.0 / np.cos(PI * d[pre + "szen"] / 180.0)
        col.solar_irrad = d[pre + "stoa"].copy()
    dtype, itype = (5, 8) if ga9 else ((3, 3) if solar else (1, 1))
    re = np.clip(f(d[pre + "re"]), sp.drop_parm_min_dim[dtype - 1], sp.drop_parm_max_dim[dtype - 1])
    ire = np.clip(f(d[pre + "ire"]), sp.ice_parm_min_dim[itype - 1], sp.ice_parm_max_dim[itype - 1])
    w = f(d[pre + "clfr"])
    col.cld = dict(n_condensed=2, type_condensed=[abi.IP_PHASE_WATER, abi.IP_PHASE_ICE], i_cloud_type=[1, 1],
                   n_cloud_type=1, i_condensed_param=[int(sp.i_drop_parm[dtype - 1]), int(sp.i_ice_parm[itype - 1])],
                   i_condensed_type=[dtype, itype],
                   condensed_mix_ratio=np.asfortranarray(np.stack([f(d[pre + "lwm"]), f(d[pre + "iwm"])], axis=2)),
                   condensed_dim_char=np.asfortranarray(np.stack([re, ire], axis=2)),
                   w_cloud=w, frac_cloud=np.asfortranarray(np.where(w > 0.0, 1.0, 0.0)[:, :, None]))
    common = dict(i_cloud=abi.IP_CLOUD_MIX_MAX, l_rescale=True, i_scatter_method=abi.IP_SCATTER_FULL,
                  i_solver=abi.IP_SOLVER_MIX_DIRECT_HOGAN if ga9 else abi.IP_SOLVER_MIX_DIRECT, l_flux_div=False,
                  precision=precision, i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL if ga9 else abi.IP_OVERLAP_RANDOM,
                  l_continuum=ga9 or not solar)
    if solar:
        ctl = R.sw_control(i_2stream=abi.IP_PIFM80 if ga9 else abi.IP_EDDINGTON, l_rayleigh=True, **common)
        if run.endswith("ds0") or run.endswith("ds0_avg"):
            ctl = replace(ctl, i_direct_tau=abi.IP_DIRECT_NOSCALING)
    else:
        ctl = R.lw_control(i_2stream=abi.IP_ELSASSER, l_ir_source_quad=False, **common)
    kgo = np.asarray(d["kgo_" + run])
    return ctl, sp, col, kgo, ("nflx" if ga9 else "hrts")


def printed(out, col, kind):
    """The quantity the known-good file holds, (columns, values)."""
    if kind == "nflx":
        return out["flux_down"] - out["flux_up"]
    return circ6.heating_rate(out, col.mass)


def half_units(got, kgo):
    """|got - kgo| in half units of the 6th significant digit of kgo."""
    kgo = np.asarray(kgo, dtype=np.float64)
    scale = 0.5 * 10.0 ** (np.floor(np.log10(np.maximum(np.abs(kgo), 1e-300))) - 5)
    return np.abs(got - kgo) / scale
