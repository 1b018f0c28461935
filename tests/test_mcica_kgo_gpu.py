"""McICA on the GPU against the reference's known-good outputs
(examples/netcdf/mcica) and the oracle: the generator's subcolumns bit for
bit, FP64 fluxes within 1e-10 of the largest flux, the printed heating rates
to half a unit of their 6th digit, mixed precision within 0.1 W/m2 and
0.05 K/day.  The ice schemes (Slingo-Schrecker, Fu), which the known-good
column does not exercise (it holds no ice), are checked against the oracle
on the same column with ice added."""
from dataclasses import replace

import numpy as np
import pytest

import circ6
import mcica5118 as M
from socrates_gb300 import abi
from socrates_gb300 import radiance as R
from test_parity_gpu import assert_fp64_parity, assert_mixed_tolerance

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def O():
    import oracle
    return oracle


@pytest.fixture(scope="module")
def sps():
    return M.spectra()


def _state(run, sps, O, ice=False, n_col=1):
    ctl, sp, col, data, kgo = M.setup(run, sps, n_col=n_col)
    if ice:
        # ice in the cloudy layers, a third of the water content plus a floor
        cmr = col.cld["condensed_mix_ratio"]
        cmr[:, :, 1] = np.where(col.cld["w_cloud"] > 0.0, cmr[:, :, 0] / 3.0 + 2.0e-5, 0.0)
    kw = dict(sampling=abi.IP_MCICA_OPTIMAL_SAMPLING, ioverlap=abi.IP_EXPONENTIAL, rng=abi.RNG_LCG, data=data)
    m_gpu = R.set_cld_mcica(sp, col, ctl.isolir, **kw)
    m_ora = R.set_cld_mcica(sp, col, ctl.isolir, impl=O.cloud_gen_impl, **kw)
    assert np.array_equal(m_gpu.c_sub, m_ora.c_sub) and np.array_equal(m_gpu.n_subcol_cld, m_ora.n_subcol_cld)
    return ctl, sp, col, m_gpu, kgo


@pytest.mark.parametrize("run", M.RUNS)
def test_mcica5118_known_good_output_on_gpu(gpu_lib, O, sps, run):
    ctl, sp, col, m, kgo = _state(run, sps, O)
    ref = O.radiance_calc(ctl, sp, col, m)
    g64 = R.radiance_calc(replace(ctl, precision=abi.PRECISION_FP64), sp, col, m)
    assert_fp64_parity({**g64, "mass": col.mass}, {**ref, "mass": col.mass}, f"{run} fp64: ")
    hr = circ6.heating_rate(g64, col.mass)[0]
    half_unit = 0.5 * 10.0 ** (np.floor(np.log10(np.abs(kgo))) - 5)
    err = np.abs(hr - kgo) / half_unit
    assert err.max() <= 1.05, f"{run} layer {err.argmax()}: {hr[err.argmax()]} vs {kgo[err.argmax()]}"
    gmx = R.radiance_calc(replace(ctl, precision=abi.PRECISION_MIXED), sp, col, m)
    assert_mixed_tolerance(gmx, {**ref, "heating_rate": circ6.heating_rate(ref, col.mass)}, f"{run} mixed: ")


@pytest.mark.parametrize("run", ["lw_avg", "sw_avg", "lw_ga7", "sw_ga7"])
def test_mcica5118_with_ice_on_gpu(gpu_lib, O, sps, run):
    """Slingo-Schrecker ice (GA3.0, type 1 and 3) and Fu's ice (GA7, type 8)
    with droplets in one homogeneous cloud type, over 64 copies of the
    column with their own seeds."""
    ctl, sp, col, m, _ = _state(run, sps, O, ice=True, n_col=64)
    ref = O.radiance_calc(ctl, sp, col, m)
    plain = O.radiance_calc(ctl, sp, *_state(run, sps, O, n_col=64)[2:4])
    assert np.abs(ref["flux_up"] - plain["flux_up"]).max() > 1e-2     # the ice matters
    g64 = R.radiance_calc(replace(ctl, precision=abi.PRECISION_FP64), sp, col, m)
    assert_fp64_parity({**g64, "mass": col.mass}, {**ref, "mass": col.mass}, f"{run} ice fp64: ")
    gmx = R.radiance_calc(replace(ctl, precision=abi.PRECISION_MIXED), sp, col, m)
    assert_mixed_tolerance(gmx, {**ref, "heating_rate": circ6.heating_rate(ref, col.mass)}, f"{run} ice mixed: ")


def test_csr_scaled_direct_beam_is_refused(gpu_lib, O, sps):
    """The direct beam scaled by the circumsolar correction (i_direct_tau = 2)
    is not built in the kernels: the call fails with i_err_fatal and a
    message."""
    ctl, sp, col, m, _ = _state("sw_avg", sps, O)
    with pytest.raises(R.RadianceError) as e:
        R.radiance_calc(replace(ctl, i_direct_tau=abi.IP_DIRECT_CSR_SCALING), sp, col, m)
    assert e.value.status == abi.I_ERR_FATAL and "i_direct_tau" in str(e.value)


@pytest.mark.parametrize("name,gas_overlap", [("hsw", abi.IP_OVERLAP_RANDOM), ("ga9sw", abi.IP_OVERLAP_K_EQV_SCL)])
def test_unscaled_direct_beam_clear_sky(gpu_lib, O, name, gas_overlap):
    """Clear sky with the direct beam not delta-scaled (i_direct_tau = 0):
    HadGEM1 shortwave with random overlap and GA9 with k_eqv_scl and the
    continuum, Rayleigh and a delta-rescaled aerosol mode, 97 columns of 60
    layers, FP64 and mixed against the oracle, and the direct flux and the
    ground's direct reflection differing from the scaled run."""
    import cld7460 as K
    from socrates_gb300 import synth
    sp = K.spectra()[name]
    col = synth.add_aerosol(synth.operational_case(sp, 97, 60, seed=67, solar=True), sp, seed=67)
    col.rho_alb[:, 1, :] = 0.55 * col.rho_alb[:, 0, :] + 0.05       # direct albedos apart from the diffuse ones
    ctl = R.sw_control(l_rayleigh=True, l_continuum=name == "ga9sw", l_aerosol_mode=True, l_rescale=True,
                       i_gas_overlap=gas_overlap, i_direct_tau=abi.IP_DIRECT_NOSCALING, l_flux_div=False)
    ref = O.radiance_calc(ctl, sp, col)
    scaled = O.radiance_calc(replace(ctl, i_direct_tau=abi.IP_DIRECT_DELTA_SCALING), sp, col)
    assert np.abs(ref["flux_direct"] - scaled["flux_direct"]).max() > 1.0
    assert np.abs(ref["flux_up"] - scaled["flux_up"]).max() > 1e-2          # the ground's direct reflection
    g64 = R.radiance_calc(replace(ctl, precision=abi.PRECISION_FP64), sp, col)
    assert_fp64_parity({**g64, "mass": col.mass}, {**ref, "mass": col.mass}, "ds0 fp64: ")
    gmx = R.radiance_calc(replace(ctl, precision=abi.PRECISION_MIXED), sp, col)
    assert_mixed_tolerance(gmx, {**ref, "heating_rate": circ6.heating_rate(ref, col.mass)}, "ds0 mixed: ")
