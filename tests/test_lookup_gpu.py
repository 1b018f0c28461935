"""Operational spectral files on the GPU: lookup-table k scaling, Wen-Yi
scaling and the equivalent-extinction gas overlap (k_eqv_scl), against the
oracle and the reference's CIRC case 6 known-good heating rates.

FP64 must match the oracle within 1e-10 of the column's largest flux; mixed
precision must stay within 0.1 W/m2 and 0.05 K/day of the oracle."""
import sys
from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
sys.path.insert(0, str(HERE.parent / "oracle"))

from socrates_gb300 import abi, synth  # noqa: E402
from socrates_gb300 import radiance as R  # noqa: E402
from socrates_gb300.spectrum import Spectrum  # noqa: E402
from test_parity_gpu import assert_fp64_parity, assert_mixed_tolerance  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = HERE / "golden"


@pytest.fixture(scope="module")
def O():
    import oracle
    return oracle


def _hr(out, mass):
    net = out["flux_down"] - out["flux_up"]
    return 8.64e+04 * (net[:, :-1] - net[:, 1:]) / (mass * 1.005e+03)


def _check(ctl, sp, col, O, tag):
    ref = O.radiance_calc(ctl, sp, col)
    g64 = R.radiance_calc(replace(ctl, precision=abi.PRECISION_FP64), sp, col)
    assert_fp64_parity({**g64, "mass": col.mass}, {**ref, "mass": col.mass}, f"{tag} fp64: ")
    # mixed precision: the heating rate the kernel returns (from each layer's
    # divergence), not a difference of FP32-accurate level fluxes, which thin
    # upper layers under a 1000 W/m2 beam would amplify
    gmx = R.radiance_calc(replace(ctl, precision=abi.PRECISION_MIXED), sp, col)
    assert_mixed_tolerance(gmx, {**ref, "heating_rate": _hr(ref, col.mass)}, f"{tag} mixed: ")
    return ref, g64, gmx


def _ga7_lw():
    return Spectrum.load_npz(GOLDEN / "circ6_lw_ga7.npz", prefix="sp_")


def _ga7_sw():
    return Spectrum.load_npz(GOLDEN / "ga7_sw_spectrum.npz")


def test_circ6_ga7_known_good_output_on_gpu(gpu_lib, O):
    """CIRC case 6 with the GA7 long-wave file (lookup tables, Wen-Yi CO2
    terms, k_eqv_scl, continuum) through the CUDA path: FP64 against the
    oracle at 1e-10 and against the reference's printed heating rates to half
    a unit of their 6th digit; mixed precision within tolerance."""
    import circ6 as K
    ctl, sp, col, kgo = K.load()
    ref, g64, _ = _check(ctl, sp, col, O, "circ6")
    hr = K.heating_rate(g64, col.mass)[0]
    half_unit = 0.5 * 10.0 ** (np.floor(np.log10(np.abs(kgo))) - 5)
    err = np.abs(hr - kgo) / half_unit
    assert err.max() <= 1.0, f"layer {err.argmax()}: {hr[err.argmax()]} vs {kgo[err.argmax()]}"


@pytest.mark.parametrize("overlap", [abi.IP_OVERLAP_K_EQV_SCL, abi.IP_OVERLAP_RANDOM])
def test_ga7_lw_synthetic_columns(gpu_lib, O, overlap):
    """257 synthetic columns of 60 layers with the GA7 long-wave file under
    both gas overlaps (random overlap gives 791 k-term products)."""
    sp = _ga7_lw()
    col = synth.operational_case(sp, 257, 60, seed=41, solar=False)
    ctl = R.lw_control(i_2stream=abi.IP_ELSASSER, l_rescale=False, l_ir_source_quad=False, l_continuum=True,
                       i_gas_overlap=overlap)
    _check(ctl, sp, col, O, f"ga7 lw overlap {overlap}")


@pytest.mark.parametrize("quad", [False, True])
def test_ga7_lw_grey_single_and_quadratic_source(gpu_lib, O, quad):
    """Single-term minor absorbers as grey absorbers (l_grey_single), with
    the linear and the quadratic infra-red source."""
    sp = _ga7_lw()
    col = synth.operational_case(sp, 64, 50, seed=43, solar=False)
    ctl = R.lw_control(l_continuum=True, l_grey_single=True, l_ir_source_quad=quad,
                       i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL)
    _check(ctl, sp, col, O, f"ga7 lw grey single quad={quad}")


def test_ga7_sw_k_eqv(gpu_lib, O):
    """The GA7 short-wave file under k_eqv_scl: minor absorbers weighted by
    the direct flux they transmit, and the direct beam of the major
    absorber's solve corrected by adjust_solar_ke; Rayleigh scattering,
    PIFM80 with delta rescaling."""
    sp = _ga7_sw()
    col = synth.operational_case(sp, 257, 70, seed=45, solar=True)
    ctl = R.sw_control(l_rayleigh=True, l_continuum=True, i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL)
    _check(ctl, sp, col, O, "ga7 sw")


def test_ga7_sw_random_overlap_too_many_products(gpu_lib):
    """Random overlap of the GA7 short-wave file needs 12096 k-term products
    in band 6, more than the device tables hold: the call fails with a
    range error and a message, and equivalent extinction still works."""
    sp = _ga7_sw()
    col = synth.operational_case(sp, 4, 20, seed=47, solar=True)
    ctl = R.sw_control(l_continuum=True, i_gas_overlap=abi.IP_OVERLAP_RANDOM)
    with pytest.raises(R.RadianceError) as e:
        R.radiance_calc(ctl, sp, col)
    assert e.value.status == abi.I_ERR_RANGE and "equivalent extinction" in str(e.value)
    R.radiance_calc(replace(ctl, i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL), sp, col)


@pytest.mark.parametrize("named", [abi.IP_OVERLAP_K_EQV_SCL, abi.IP_OVERLAP_RANDOM])
def test_hybrid_overlap_takes_the_bands_method(gpu_lib, named):
    """ip_overlap_hybrid (radiance_calc.F90:888-893): when every band of the
    call names one method in the spectral file, the fluxes are that method's
    bit for bit; bands naming different methods are refused with a message,
    and a band range over which they agree runs."""
    base = _ga7_lw()
    col = synth.operational_case(base, 16, 40, seed=49, solar=False)
    ctl = R.lw_control(l_continuum=True, i_gas_overlap=named)
    hybrid = replace(ctl, i_gas_overlap=abi.IP_OVERLAP_HYBRID)
    sp = replace(base, i_overlap=np.full(base.n_band, named, np.int32), name=f"{base.name}_hybrid{named}")
    want, got = R.radiance_calc(ctl, base, col), R.radiance_calc(hybrid, sp, col)
    for k in ("flux_up", "flux_down", "heating_rate"):
        assert np.array_equal(got[k], want[k]), k
    other = abi.IP_OVERLAP_RANDOM + abi.IP_OVERLAP_K_EQV_SCL - named
    mixed = np.full(base.n_band, named, np.int32)
    mixed[-1] = other
    sp2 = replace(base, i_overlap=mixed, name=f"{base.name}_hybrid{named}_mixed")
    with pytest.raises(R.RadianceError) as e:
        R.radiance_calc(hybrid, sp2, col)
    assert e.value.status == abi.I_ERR_FATAL and "ip_overlap_hybrid" in str(e.value)
    nb = base.n_band - 1
    got = R.radiance_calc(replace(hybrid, last_band=nb), sp2, col)
    want = R.radiance_calc(replace(ctl, last_band=nb), base, col)
    assert np.array_equal(got["flux_up"], want["flux_up"]) and np.array_equal(got["flux_down"], want["flux_down"])


def _self_broadened(sp):
    """GA7 long wave with water vapour made self-broadened: three gas
    fractions, k growing with the fraction."""
    n_tmp, n_pre, nk, na, nb = sp.k_lookup.shape
    iw = int(sp.index_water) - 1
    sp.index_sb = np.zeros(na, np.int32)
    sp.index_sb[iw] = 1
    sp.gf_lookup = np.array([0.0, 0.01, 0.04])
    ksb = np.zeros((n_tmp, n_pre, 3, nk, 1, nb))
    for ig in range(3):
        ksb[:, :, ig, :, 0, :] = sp.k_lookup[:, :, :, iw, :] * (1.0 + 2.0 * ig)
    # 7 significant digits, as the '_k' file records them (1PE13.6)
    ksb = np.array([float(f"{v:.6E}") for v in ksb.ravel(order="F")]).reshape(ksb.shape, order="F")
    sp.k_lookup_sb = np.asfortranarray(ksb)
    return sp


def _temperature_tables(sp):
    """GA7 long wave with methane given temperature-only tables, taken from
    its P/T tables at one pressure."""
    n_tmp, n_pre, nk, na, nb = sp.k_lookup.shape
    ich4 = int(np.where(sp.type_absorb == 6)[0][0])
    ip = 40
    sp.n_t_lookup_gas = np.zeros(na, np.int32)
    sp.n_t_lookup_gas[ich4] = n_tmp
    tg = np.zeros((n_tmp, na))
    tg[:, ich4] = sp.t_lookup[:, ip]
    sp.t_lookup_gas = np.asfortranarray(tg)
    kt = np.zeros((n_tmp, nk, na, nb))
    kt[:, :, ich4, :] = sp.k_lookup[:, ip, :, ich4, :]
    sp.k_t_lookup_gas = np.asfortranarray(kt)
    for b in range(nb):
        if sp.i_scale_fnc[b, ich4] == abi.IP_SCALE_LOOKUP:
            sp.i_scale_fnc[b, ich4] = abi.IP_SCALE_T_LOOKUP
    return sp


@pytest.mark.parametrize("kind", ["self_broadened", "temperature_tables"])
@pytest.mark.parametrize("overlap", [abi.IP_OVERLAP_K_EQV_SCL, abi.IP_OVERLAP_RANDOM])
def test_self_broadened_and_temperature_tables(gpu_lib, O, kind, overlap):
    """Self-broadened lookup tables (gas-fraction interpolation) and
    temperature-only tables on the GPU against the oracle."""
    sp = (_self_broadened if kind == "self_broadened" else _temperature_tables)(_ga7_lw())
    sp.name = f"sp_lw_ga7_{kind}"     # spectra are registered on the device by name
    col = synth.operational_case(sp, 129, 40, seed=49, solar=False)
    ctl = R.lw_control(l_continuum=True, i_gas_overlap=overlap)
    ref, _, _ = _check(ctl, sp, col, O, f"{kind} overlap {overlap}")
    # the modified tables change the result: the feature is exercised
    plain = O.radiance_calc(ctl, _ga7_lw(), col)
    assert np.abs(plain["flux_up"] - ref["flux_up"]).max() > 1e-4
