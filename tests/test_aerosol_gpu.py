"""GPU parity of the classic aerosol species (opt_prop_aerosol.F90:273-640,
called from grey_opt_prop.F90:719-740): dry and moist species, Henyey-
Greenstein and tabulated phase-function moments, inactive and repeated
entries, humidities at the table's ends, through the C-ABI against the FP64
oracle.  Tolerances as in test_parity_gpu.py: FP64 fluxes within 1e-10 of
the column's largest flux; mixed precision within 0.1 W/m2 and 0.05 K/day."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from socrates_gb300 import abi, synth
from socrates_gb300 import radiance as R
from test_parity_gpu import assert_fp64_parity, assert_mixed_tolerance

pytestmark = pytest.mark.gpu

SOURCES = [abi.IP_AERSRC_CLASSIC_RON, abi.IP_AERSRC_CLASSIC_RON + 10, abi.IP_AERSRC_CLASSIC_RON,
           abi.IP_AERSRC_CUSACK_RON, abi.IP_AERSRC_ARCL_RON]
ENTRIES = (1, 2, 3, 4, 1)


def _case(solar, n=40, L=70, seed=61):
    if solar:
        sp, col = synth.config2(n, L, seed=seed)
    else:
        sp, col = synth.config1(n, L, seed=seed)
    col.aer = None
    synth.add_aerosol_species(sp, seed, n_humidity=21, n_phf=3)
    synth.add_aerosol_mix(col, seed, entries=ENTRIES, sources=SOURCES)
    return sp, col


def _both(ctl, sp, col):
    return ({**R.radiance_calc(ctl, sp, col), "mass": col.mass},
            {**O.radiance_calc(ctl, sp, col), "mass": col.mass})


@pytest.mark.parametrize("hg", [False, True], ids=["tabulated", "hg"])
@pytest.mark.parametrize("solar", [False, True], ids=["lw", "sw"])
def test_classic_aerosol_fp64(kernel, solar, hg):
    sp, col = _case(solar)
    mk = R.sw_control if solar else R.lw_control
    gpu, ref = _both(mk(l_aerosol=True, l_henyey_greenstein_pf=hg), sp, col)
    assert_fp64_parity(gpu, ref, f"{kernel} {'sw' if solar else 'lw'}: ")


@pytest.mark.parametrize("solar", [False, True], ids=["lw", "sw"])
def test_classic_aerosol_mixed(kernel, solar):
    sp, col = _case(solar, seed=62)
    mk = R.sw_control if solar else R.lw_control
    gpu, ref = _both(mk(l_aerosol=True, precision=abi.PRECISION_MIXED), sp, col)
    assert_mixed_tolerance(gpu, ref, f"{kernel}: ")


def test_classic_with_modal_aerosol_and_eddington(gpu_lib):
    """Classic species and a UKCA mode in the same layers, Eddington
    coefficients, humidities of exactly 0 and 1 everywhere in two columns."""
    sp, col = synth.config2(24, 90, seed=63)
    synth.add_aerosol_species(sp, 63)
    synth.add_aerosol_mix(col, 63, entries=(4, 1, 2))
    col.aer["mean_rel_humidity"][0, :] = 0.0
    col.aer["mean_rel_humidity"][1, :] = 1.0
    ctl = R.sw_control(i_2stream=abi.IP_EDDINGTON, l_aerosol=True, l_aerosol_mode=True)
    gpu, ref = _both(ctl, sp, col)
    assert_fp64_parity(gpu, ref, "classic+modal: ")


def test_loader_reads_aerosol_block(gpu_lib, tmp_path):
    """The species written as spectral-file block 11 and read by the C++
    loader (socgpu_spectrum_load) solve to the oracle's fluxes on the
    tables read back by the Python reader."""
    from socrates_gb300.spectrum import Spectrum
    sp, col = _case(True, n=16, L=50, seed=64)
    path = tmp_path / "sp_sw_aer"
    sp.write_text(path)
    back = Spectrum.read_text(path)
    lib = R.load_library()
    h = C.c_int(0)
    msg = C.create_string_buffer(512)
    st = lib.socgpu_spectrum_load(b"loaded_aerosol", str(path).encode(), C.byref(h), msg, 512)
    assert st == 0, msg.value.decode()
    ctl = R.sw_control(l_aerosol=True)
    m = R.Marshal(ctl, back, col)
    st = lib.socgpu_radiance_calc(*m.args(h.value), msg, 512)
    assert st == 0, msg.value.decode()
    got = {**m.result(), "mass": col.mass}
    ref = {**O.radiance_calc(ctl, back, col), "mass": col.mass}
    assert_fp64_parity(got, ref, "loaded: ")


def test_classic_aerosol_inputs_are_checked(gpu_lib):
    sp, col = _case(False, n=4, L=30)
    col.aer["mr_type_index"] = np.array([1, 2, 3, 9, 1], np.int32)
    with pytest.raises(R.RadianceError, match="species"):
        R.radiance_calc(R.lw_control(l_aerosol=True), sp, col)
    sp, col = _case(False, n=4, L=30)
    col.aer["mean_rel_humidity"] = None
    with pytest.raises(R.RadianceError, match="humidit"):
        R.radiance_calc(R.lw_control(l_aerosol=True), sp, col)
    sp, col = _case(False, n=4, L=30)
    sp.type_aerosol = sp.i_aerosol_parm = sp.nhumidity = sp.n_aerosol_phf_term = None
    sp.aerosol_humidities = sp.aerosol_abs = sp.aerosol_scat = sp.aerosol_phf = None
    sp.name += "_without_species"
    with pytest.raises(R.RadianceError, match="aerosol"):
        R.radiance_calc(R.lw_control(l_aerosol=True), sp, col)


def test_classic_aerosol_with_mcica_clouds(gpu_lib):
    """Classic species in the clear-sky optics beneath McICA clouds: the
    cloudy sub-columns start from the same aerosol phase moments."""
    from oracle import cloud_gen_impl
    lw, sw, col = synth.config3(16, 85, seed=65, n_subcol=16)
    synth.add_sw_surface(col, sw.n_band, 65)
    synth.add_aerosol_species(sw, 65)
    synth.add_aerosol_mix(col, 65)
    ctl = R.sw_control(i_cloud=abi.IP_CLOUD_MCICA, l_aerosol=True)
    c_sub, nsc = R.cloud_gen(col, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_LCG, impl=cloud_gen_impl)
    mc = R.set_cld_mcica(sw, col, abi.IP_SOLAR, abi.IP_MCICA_SINGLE_SAMPLING, c_sub=c_sub, n_subcol_cld=nsc)
    gpu = {**R.radiance_calc(ctl, sw, col, mc), "mass": col.mass}
    ref = {**O.radiance_calc(ctl, sw, col, mc), "mass": col.mass}
    assert_fp64_parity(gpu, ref, "mcica: ")


def _prsc_case(solar, n=40, L=70, seed=66, n_phf=2):
    if solar:
        sp, col = synth.config2(n, L, seed=seed)
    else:
        sp, col = synth.config1(n, L, seed=seed)
    col.aer = None
    synth.add_density(col, 1)
    synth.add_aerosol_species(sp, seed, n_humidity=21, n_phf=3)
    # species 2 prescribed, named by an inactive entry and an active one;
    # the others parametrized
    synth.add_aerosol_mix(col, seed, entries=(1, 2, 3, 2, 4), sources=SOURCES)
    return synth.add_prescribed_aerosol(sp, col, seed, species=(2,), n_phf=n_phf)


@pytest.mark.parametrize("hg", [False, True], ids=["tabulated", "hg"])
@pytest.mark.parametrize("solar", [False, True], ids=["lw", "sw"])
def test_prescribed_aerosol_fp64(kernel, solar, hg):
    """Prescribed optical properties (prsc_opt_prop.F90) of one species next
    to parametrized ones: the spline kernel and the flux kernels against the
    oracle."""
    sp, col = _prsc_case(solar)
    mk = R.sw_control if solar else R.lw_control
    gpu, ref = _both(mk(l_aerosol=True, l_henyey_greenstein_pf=hg), sp, col)
    assert_fp64_parity(gpu, ref, f"{kernel} prescribed: ")


@pytest.mark.parametrize("solar", [False, True], ids=["lw", "sw"])
def test_prescribed_aerosol_mixed(kernel, solar):
    sp, col = _prsc_case(solar, seed=67)
    mk = R.sw_control if solar else R.lw_control
    gpu, ref = _both(mk(l_aerosol=True, l_henyey_greenstein_pf=True, precision=abi.PRECISION_MIXED), sp, col)
    assert_mixed_tolerance(gpu, ref, f"{kernel} prescribed: ")


def test_prescribed_aerosol_in_column_windows(gpu_lib):
    """Enough columns that the host path copies and solves them in several
    windows: the prescribed arrays move with each window."""
    sp, col = _prsc_case(True, n=1500, L=40, seed=68)
    gpu, ref = _both(R.sw_control(l_aerosol=True, l_henyey_greenstein_pf=True), sp, col)
    assert_fp64_parity(gpu, ref, "windows: ")


def test_prescribed_aerosol_checks(gpu_lib):
    from socrates_gb300.server import Server
    sp, col = _prsc_case(False, n=6, L=30, seed=69)
    # moments: the tabulated forward moment needs n_order_forward (2) of them
    col.aer["n_phase_term_prsc"] = np.ones_like(col.aer["n_phase_term_prsc"])
    with pytest.raises(R.RadianceError, match="moments"):
        R.radiance_calc(R.lw_control(l_aerosol=True), sp, col)
    sp, col = _prsc_case(False, n=6, L=30, seed=69)
    col.density = None
    with pytest.raises(R.RadianceError, match="density"):
        R.radiance_calc(R.lw_control(l_aerosol=True), sp, col)
    sp, col = _prsc_case(False, n=6, L=30, seed=69)
    R.register_spectrum(sp)
    srv = Server(device_bytes=64 << 20, streams=1)
    with pytest.raises(R.RadianceError, match="server"):
        srv.submit(R.Marshal(R.lw_control(l_aerosol=True), sp, col), sp)
    srv.close()


def test_circ6_sw_aerosol_known_good_output(gpu_lib, kernel):
    """The reference's CIRC case 6 short-wave run with prescribed soot and
    two-region clouds (ref_case6_sw_ga7.hrts) on the GPU: FP64 within 1e-10
    of the oracle and within half a unit of the 6th significant digit of the
    known-good heating rates (5 % slack on rounding boundaries); mixed
    precision within its tolerance of the oracle."""
    import circ6_sw as K
    from cld7460 import half_units
    ctl, sp, col, kgo = K.load()
    gpu, ref = _both(ctl, sp, col)
    assert_fp64_parity(gpu, ref, f"{kernel} circ6 sw: ")
    hr = K.heating_rate(gpu, col)[0]
    err = half_units(hr, kgo)
    assert err.max() <= 1.05, f"layer {err.argmax()}: {hr[err.argmax()]} vs {kgo[err.argmax()]}"
    from dataclasses import replace
    ctl_m = replace(ctl, precision=abi.PRECISION_MIXED)
    gpu_m, ref_m = _both(ctl_m, sp, col)
    assert_mixed_tolerance(gpu_m, ref, f"{kernel} circ6 sw mixed: ")
