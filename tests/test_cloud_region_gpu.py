"""Clouds in a clear and a cloudy region (ip_cloud_mix_max / mix_random with
solver_mix_direct and Hogan's form) on the GPU: the reference's 7460_28
known-good outputs, FP64 against the oracle within 1e-10 of the largest flux,
mixed precision within 0.1 W/m2 and 0.05 K/day; synthetic columns over both
overlaps, both solvers, both cloud representations and both sources."""
from dataclasses import replace

import numpy as np
import pytest

import cld7460 as K
from socrates_gb300 import abi, synth
from socrates_gb300 import radiance as R
from test_parity_gpu import assert_fp64_parity, assert_mixed_tolerance

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def O():
    import oracle
    return oracle


@pytest.fixture(scope="module")
def sps():
    return K.spectra()


def _check(ctl, sp, col, O, tag):
    ref = O.radiance_calc(ctl, sp, col)
    g64 = R.radiance_calc(replace(ctl, precision=abi.PRECISION_FP64), sp, col)
    assert_fp64_parity({**g64, "mass": col.mass}, {**ref, "mass": col.mass}, f"{tag} fp64: ")
    gmx = R.radiance_calc(replace(ctl, precision=abi.PRECISION_MIXED), sp, col)
    net = ref["flux_down"] - ref["flux_up"]
    hr = 8.64e+04 * (net[:, :-1] - net[:, 1:]) / (col.mass * 1.005e+03)
    assert_mixed_tolerance(gmx, {**ref, "heating_rate": hr}, f"{tag} mixed: ")
    return ref, g64


@pytest.mark.parametrize("run", K.RUNS)
def test_cloud_regions_known_good_output_on_gpu(gpu_lib, O, sps, run):
    ctl, sp, col, kgo, kind = K.setup(run, sps)
    _, g64 = _check(ctl, sp, col, O, run)
    got = K.printed(g64, col, kind)
    got = got[0] if kgo.ndim == 1 else got.T
    err = K.half_units(got, kgo)
    i = np.unravel_index(err.argmax(), err.shape)
    assert err.max() <= 1.05, f"{run} at {i}: {got[i]} vs {kgo[i]}"


def _clouded(sp, n, L, seed, solar, representation):
    """operational_case columns with cloud layers of water and ice."""
    col = synth.operational_case(sp, n, L, seed=seed, solar=solar)
    rng = np.random.default_rng(seed)
    w = np.where(rng.uniform(size=(n, L)) < 0.35, rng.uniform(0.05, 1.0, size=(n, L)), 0.0)
    w[:, : L // 4] = 0.0                                   # clear stratosphere
    lwm = np.where(w > 0, rng.uniform(1e-5, 5e-4, size=(n, L)), 0.0)
    iwm = np.where(w > 0, rng.uniform(0.0, 2e-4, size=(n, L)), 0.0)
    f = lambda a: np.asfortranarray(a)
    dtype, itype = 5, 8
    re = np.clip(rng.uniform(4e-6, 2e-5, size=(n, L)), sp.drop_parm_min_dim[dtype - 1], sp.drop_parm_max_dim[dtype - 1])
    ire = np.clip(rng.uniform(2e-5, 1e-4, size=(n, L)), sp.ice_parm_min_dim[itype - 1], sp.ice_parm_max_dim[itype - 1])
    cld = dict(n_condensed=2, type_condensed=[abi.IP_PHASE_WATER, abi.IP_PHASE_ICE],
               i_condensed_param=[int(sp.i_drop_parm[dtype - 1]), int(sp.i_ice_parm[itype - 1])],
               i_condensed_type=[dtype, itype], condensed_mix_ratio=f(np.stack([lwm, iwm], axis=2)),
               condensed_dim_char=f(np.stack([re, ire], axis=2)), w_cloud=f(w))
    if representation == abi.IP_CLOUD_HOMOGEN:
        cld.update(i_cloud_type=[1, 1], n_cloud_type=1, frac_cloud=f(np.where(w > 0, 1.0, 0.0)[:, :, None]))
    else:
        fw = np.where(w > 0, rng.uniform(0.2, 0.8, size=(n, L)), 0.0)
        cld.update(i_cloud_type=[1, 2], n_cloud_type=2, frac_cloud=f(np.stack([fw, np.where(w > 0, 1.0 - fw, 0.0)],
                                                                               axis=2)))
    col.cld = cld
    return col


@pytest.mark.parametrize("solar", [False, True])
@pytest.mark.parametrize("scheme,solver,representation", [
    (abi.IP_CLOUD_MIX_MAX, abi.IP_SOLVER_MIX_DIRECT, abi.IP_CLOUD_HOMOGEN),
    (abi.IP_CLOUD_MIX_MAX, abi.IP_SOLVER_MIX_DIRECT_HOGAN, abi.IP_CLOUD_ICE_WATER),
    (abi.IP_CLOUD_MIX_RANDOM, abi.IP_SOLVER_MIX_DIRECT, abi.IP_CLOUD_ICE_WATER),
    (abi.IP_CLOUD_MIX_RANDOM, abi.IP_SOLVER_MIX_DIRECT_HOGAN, abi.IP_CLOUD_HOMOGEN)])
def test_cloud_regions_synthetic(gpu_lib, O, sps, solar, scheme, solver, representation):
    """97 columns of 60 layers with the GA9 files, k_eqv_scl and continuum:
    random cloud layers of water (Pade) and ice (Fu) as one type or as two."""
    sp = sps["ga9sw" if solar else "ga9lw"]
    col = _clouded(sp, 97, 60, seed=61 + solar, solar=solar, representation=representation)
    common = dict(i_cloud=scheme, i_solver=solver, l_continuum=True, i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL,
                  l_flux_div=False)
    ctl = R.sw_control(l_rayleigh=True, **common) if solar else R.lw_control(l_ir_source_quad=True, **common)
    ref, _ = _check(ctl, sp, col, O, f"{scheme}/{solver}/{representation} solar={solar}")
    clear = O.radiance_calc(replace(ctl, i_cloud=abi.IP_CLOUD_CLEAR, i_solver=abi.IP_SOLVER_HOMOGEN_DIRECT), sp, col)
    assert np.abs(ref["flux_up"] - clear["flux_up"]).max() > 1.0          # the clouds matter


def test_cloud_regions_refusals(gpu_lib, sps):
    """A solver of another scheme is refused."""
    ctl, sp, col, _, _ = K.setup("sw_avg", sps)
    with pytest.raises(R.RadianceError) as e:
        R.radiance_calc(replace(ctl, i_solver=abi.IP_SOLVER_HOMOGEN_DIRECT), sp, col)
    assert e.value.status == abi.I_ERR_FATAL and "solver_mix" in str(e.value)


def _three_region(sp, n, L, seed, solar, representation):
    """_clouded columns whose water and ice are split between a stratiform and
    a convective part (the convective one denser): four cloud types under
    csiw (stratiform water and ice, convective water and ice), or two under
    conv_strat (each type holding a water and an ice component)."""
    col = _clouded(sp, n, L, seed, solar, abi.IP_CLOUD_ICE_WATER)
    c = col.cld
    rng = np.random.default_rng(seed + 100)
    w = c["w_cloud"]
    x = np.where(w > 0, rng.uniform(0.2, 0.8, size=w.shape), 0.0)          # the stratiform share
    fw = c["frac_cloud"][:, :, 0]                                           # the water share
    mr, dc = c["condensed_mix_ratio"], c["condensed_dim_char"]
    f = lambda a: np.asfortranarray(a)
    cld = dict(c)
    cld.update(n_condensed=4, type_condensed=[abi.IP_CLCMP_ST_WATER, abi.IP_CLCMP_ST_ICE, abi.IP_CLCMP_CNV_WATER,
                                              abi.IP_CLCMP_CNV_ICE],
               i_condensed_param=list(c["i_condensed_param"]) * 2, i_condensed_type=list(c["i_condensed_type"]) * 2,
               condensed_mix_ratio=f(np.concatenate([mr, mr * np.array([2.0, 1.5])], axis=2)),
               condensed_dim_char=f(np.concatenate([dc, dc], axis=2)))
    if representation == abi.IP_CLOUD_CSIW:
        cld.update(i_cloud_type=[abi.IP_CLOUD_TYPE_SW, abi.IP_CLOUD_TYPE_SI, abi.IP_CLOUD_TYPE_CW, abi.IP_CLOUD_TYPE_CI],
                   n_cloud_type=4,
                   frac_cloud=f(np.stack([fw * x, (1 - fw) * x * (w > 0), fw * (1 - x), (1 - fw) * (1 - x) * (w > 0)],
                                         axis=2)))
    else:
        cld.update(i_cloud_type=[abi.IP_CLOUD_TYPE_STRAT, abi.IP_CLOUD_TYPE_STRAT, abi.IP_CLOUD_TYPE_CONV,
                                 abi.IP_CLOUD_TYPE_CONV],
                   n_cloud_type=2, frac_cloud=f(np.stack([x, np.where(w > 0, 1.0 - x, 0.0)], axis=2)))
    col.cld = cld
    return col


def _three_region_control(solar, representation, **kw):
    common = dict(i_cloud=abi.IP_CLOUD_TRIPLE, i_solver=abi.IP_SOLVER_TRIPLE_HOGAN, l_continuum=True,
                  i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL, l_flux_div=False, i_cloud_representation=representation)
    common.update(kw)
    return R.sw_control(l_rayleigh=True, **common) if solar else R.lw_control(l_ir_source_quad=True, **common)


@pytest.mark.parametrize("solar", [False, True])
@pytest.mark.parametrize("representation", [abi.IP_CLOUD_CSIW, abi.IP_CLOUD_CONV_STRAT])
def test_three_regions_synthetic(gpu_lib, O, sps, solar, representation):
    """Clouds in three regions, clear, stratiform and convective (ip_cloud_triple,
    triple_column.F90, solver_triple_hogan.F90): 97 columns of 60 layers with the
    GA9 files, k_eqv_scl and continuum, the cloud split at random between a
    stratiform and a denser convective part.  FP64 within 1e-10 of the oracle,
    mixed within 0.1 W/m2 and 0.05 K/day; the split changes the answer of one
    cloudy region."""
    sp = sps["ga9sw" if solar else "ga9lw"]
    col = _three_region(sp, 97, 60, seed=71 + solar, solar=solar, representation=representation)
    ctl = _three_region_control(solar, representation)
    ref, _ = _check(ctl, sp, col, O, f"triple {representation} solar={solar}")
    one = _clouded(sp, 97, 60, seed=71 + solar, solar=solar, representation=abi.IP_CLOUD_ICE_WATER)
    two = O.radiance_calc(replace(ctl, i_cloud=abi.IP_CLOUD_MIX_MAX, i_solver=abi.IP_SOLVER_MIX_DIRECT_HOGAN,
                                  i_cloud_representation=abi.IP_CLOUD_ICE_WATER), sp, one)
    assert np.abs(ref["flux_up"] - two["flux_up"]).max() > 0.5


@pytest.mark.parametrize("solar", [False, True])
@pytest.mark.parametrize("three", [False, True])
def test_partially_correlated_regions(gpu_lib, O, sps, solar, three):
    """Like regions correlated over a pressure scale (ip_cloud_part_corr with
    two regions, ip_cloud_part_corr_cnv with three; overlap_coupled.F90:
    209-236): exp(dp / dp_corr) at each interior interface, 1 Pa for the clear
    region, 3000 Pa stratiform and 1000 Pa convective.  FP64 within 1e-10 of
    the oracle and mixed within tolerance; the answer lies apart from both
    maximal and random overlap."""
    sp = sps["ga9sw" if solar else "ga9lw"]
    if three:
        col = _three_region(sp, 97, 60, seed=91 + solar, solar=solar, representation=abi.IP_CLOUD_CSIW)
        ctl = _three_region_control(solar, abi.IP_CLOUD_CSIW, i_cloud=abi.IP_CLOUD_PART_CORR_CNV)
    else:
        col = _clouded(sp, 97, 60, seed=91 + solar, solar=solar, representation=abi.IP_CLOUD_ICE_WATER)
        common = dict(i_cloud=abi.IP_CLOUD_PART_CORR, i_solver=abi.IP_SOLVER_MIX_DIRECT_HOGAN, l_continuum=True,
                      i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL, l_flux_div=False)
        ctl = R.sw_control(l_rayleigh=True, **common) if solar else R.lw_control(l_ir_source_quad=True, **common)
    col.cld = dict(col.cld, dp_corr_strat=3000.0, dp_corr_conv=1000.0)
    ref, _ = _check(ctl, sp, col, O, f"part_corr three={three} solar={solar}")
    for other in ((abi.IP_CLOUD_TRIPLE,) if three else (abi.IP_CLOUD_MIX_MAX, abi.IP_CLOUD_MIX_RANDOM)):
        alt = O.radiance_calc(replace(ctl, i_cloud=other), sp, col)
        assert np.abs(ref["flux_up"] - alt["flux_up"]).max() > 0.05, other


def test_three_regions_unscaled_direct_beam(gpu_lib, O, sps):
    """The solar direct beam without delta-scaling (i_direct_tau = 0) through
    the three regions (triple_solar_source.F90:300-350)."""
    sp = sps["ga9sw"]
    col = _three_region(sp, 61, 60, seed=83, solar=True, representation=abi.IP_CLOUD_CSIW)
    _check(_three_region_control(True, abi.IP_CLOUD_CSIW, i_direct_tau=abi.IP_DIRECT_NOSCALING), sp, col, O,
           "triple unscaled beam")


def test_three_regions_refusals(gpu_lib, sps):
    """ip_cloud_triple needs solver_triple_hogan and a representation that
    separates convective from stratiform cloud (aggregate_cloud.F90:155-160)."""
    sp = sps["ga9lw"]
    col = _three_region(sp, 4, 60, seed=5, solar=False, representation=abi.IP_CLOUD_CSIW)
    for kw, text in ((dict(i_solver=abi.IP_SOLVER_MIX_DIRECT_HOGAN), "solver_triple_hogan"),
                     (dict(i_cloud_representation=abi.IP_CLOUD_ICE_WATER), "not compatible")):
        with pytest.raises(R.RadianceError) as e:
            R.radiance_calc(_three_region_control(False, abi.IP_CLOUD_CSIW, **kw), sp, col)
        assert e.value.status == abi.I_ERR_FATAL and text in str(e.value)
