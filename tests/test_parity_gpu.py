"""GPU parity: the CUDA path through the C-ABI against the FP64 oracle.

Tolerances (written here, per the path's contract):
  * FP64 device kernels: fluxes within 1e-10 relative of the oracle (scaled
    by the column's largest flux), heating rates within 1e-9 of the
    column's largest magnitude;
  * mixed FP32/FP64 kernels: fluxes within 0.1 W/m2, heating rates within
    0.05 K/day;
  * McICA subcolumn masks: bit-exact.
"""
import copy

import numpy as np
import pytest

import oracle as O
from golden_cases import CASES
from socrates_gb300 import abi, synth
from socrates_gb300 import radiance as R

pytestmark = pytest.mark.gpu

FLUX_KEYS = ("flux_up", "flux_down", "flux_direct")


def _gpu(ctl, sp, col, mc=None):
    return {**R.radiance_calc(ctl, sp, col, mc), "mass": col.mass}


def _ora(ctl, sp, col, mc=None):
    return {**O.radiance_calc(ctl, sp, col, mc), "mass": col.mass}


def assert_fp64_parity(gpu, ref, tag="", mass=None):
    """Fluxes within 1e-10 of the column's largest flux.  The flux
    divergence and heating rate are differences of fluxes, so their
    tolerance is that flux tolerance carried through their own formulas
    (two levels; heating rate = 86400 div / (mass cp))."""
    fscale = np.maximum.reduce([np.abs(ref[k]).max(axis=1) for k in FLUX_KEYS if k in ref])[:, None] + 1e-300
    for k in ref:
        if k == "mass":
            continue
        g, r = gpu[k], ref[k]
        if k in FLUX_KEYS:
            err = np.abs(g - r) / fscale
            assert err.max() <= 1e-10, f"{tag}{k}: max scaled error {err.max():.3e}"
        elif k == "flux_div":
            err = np.abs(g - r) / (2e-10 * fscale)
            assert err.max() <= 1.0, f"{tag}{k}: error {err.max():.3e} x tolerance"
        elif k == "heating_rate":
            m = ref.get("mass", mass)
            tol = 2e-10 * fscale * 8.64e4 / (m * 1.005e3)
            err = np.abs(g - r) / tol
            assert err.max() <= 1.0, f"{tag}{k}: error {err.max():.3e} x tolerance"


def assert_mixed_tolerance(gpu, ref, tag=""):
    for k in FLUX_KEYS:
        if k in ref:
            err = np.abs(gpu[k] - ref[k]).max()
            assert err <= 0.1, f"{tag}{k}: max error {err:.4f} W/m2"
    err = np.abs(gpu["heating_rate"] - ref["heating_rate"]).max()
    assert err <= 0.05, f"{tag}heating_rate: max error {err:.4f} K/day"


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_matches_oracle(gpu_lib, name):
    gpu = CASES[name](_gpu)
    ref = CASES[name](_ora)
    assert_fp64_parity(gpu, ref, f"{name}: ")


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_matches_golden_fixture(gpu_lib, name):
    from pathlib import Path
    data = np.load(Path(__file__).resolve().parent / "golden" / f"{name}.npz")
    gpu = CASES[name](_gpu)
    assert_fp64_parity(gpu, {k: data[k] for k in data.files}, f"{name}: ", mass=gpu["mass"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_mixed_within_tolerance(gpu_lib, name):
    gpu = CASES[name](lambda c, s, col, mc=None: _gpu(_with(c, abi.PRECISION_MIXED), s, col, mc))
    ref = CASES[name](_ora)
    assert_mixed_tolerance(gpu, ref, f"{name}: ")


def test_results_are_deterministic(gpu_lib):
    for prec in (abi.PRECISION_FP64, abi.PRECISION_MIXED):
        a = CASES["sw_pifm80"](lambda c, s, col, mc=None: _gpu(_with(c, prec), s, col, mc))
        b = CASES["sw_pifm80"](lambda c, s, col, mc=None: _gpu(_with(c, prec), s, col, mc))
        for k in a:
            np.testing.assert_array_equal(a[k], b[k])


def _with(c, prec):
    from dataclasses import replace
    return replace(c, precision=prec)


@pytest.mark.parametrize("ioverlap", [abi.IP_MAX_RAND, abi.IP_RAND, abi.IP_EXPONENTIAL, abi.IP_EXPONENTIAL_RAND])
@pytest.mark.parametrize("rng", [abi.RNG_LCG, abi.RNG_PHILOX])
def test_cloud_gen_masks_bit_exact(gpu_lib, ioverlap, rng):
    lw, sw, col = synth.config3(512, 85, seed=7, n_subcol=16)
    g, gn = R.cloud_gen(col, 16, ioverlap, rng)
    o, on = R.cloud_gen(col, 16, ioverlap, rng, impl=O.cloud_gen_impl)
    np.testing.assert_array_equal(gn, on)
    np.testing.assert_array_equal(g, o)
    assert gn.max() > 0


def test_philox_masks_independent_of_batch(gpu_lib):
    """A column's Philox subcolumns depend only on its own seed and fields."""
    lw, sw, col = synth.config3(64, 60, seed=8, n_subcol=16)
    full, nf = R.cloud_gen(col, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_PHILOX)
    sub = _subset(col, np.arange(10, 20))
    part, npart = R.cloud_gen(sub, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_PHILOX)
    np.testing.assert_array_equal(part, full[10:20])
    np.testing.assert_array_equal(npart, nf[10:20])


def _subset(col, idx):
    c = copy.copy(col)
    c.n_profile = len(idx)
    for name in ("p", "t", "p_level", "t_level", "mass", "gas_mix_ratio", "z", "t_ground", "zen_0", "solar_irrad",
                 "rho_alb"):
        v = getattr(col, name)
        if v is not None:
            setattr(c, name, np.asfortranarray(v[idx]))
    if col.aer:
        c.aer = {k: (np.asfortranarray(v[idx]) if isinstance(v, np.ndarray) else v) for k, v in col.aer.items()}
    if col.cld:
        c.cld = {k: (np.asfortranarray(v[idx]) if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == col.n_profile
                     else v) for k, v in col.cld.items()}
    return c


def test_full_size_shortwave_properties(gpu_lib):
    """10 000 columns x 100 layers: FP64 device path against the oracle on a
    sample of columns, mixed path against FP64 everywhere, energy balance."""
    sp, col = synth.config2(10000, 100, seed=2)
    ctl = R.sw_control(l_aerosol_mode=True)
    g64 = R.radiance_calc(ctl, sp, col)
    gmx = R.radiance_calc(_with(ctl, abi.PRECISION_MIXED), sp, col)
    idx = np.random.default_rng(0).choice(col.n_profile, 48, replace=False)
    ref = O.radiance_calc(ctl, sp, _subset(col, idx))
    assert_fp64_parity({k: v[idx] for k, v in g64.items()}, ref, "sample: ", mass=col.mass[idx])
    assert_mixed_tolerance(gmx, g64, "mixed vs fp64: ")
    # energy: TOA incoming = reflected + absorbed in the column + absorbed at the surface
    toa_in = col.solar_irrad * sp.solar_flux_band.sum() / col.zen_0
    np.testing.assert_allclose(g64["flux_down"][:, 0], toa_in, rtol=1e-12)
    absorbed = g64["flux_div"].sum(axis=1)
    net_toa = g64["flux_down"][:, 0] - g64["flux_up"][:, 0]
    net_sfc = g64["flux_down"][:, -1] - g64["flux_up"][:, -1]
    np.testing.assert_allclose(absorbed, net_toa - net_sfc, rtol=1e-8, atol=1e-8)


def test_unsupported_options_return_status(gpu_lib):
    sp, col = synth.config1(4, 20)
    bad = [
        (R.lw_control(i_2stream=abi.IP_IFM), abi.I_ERR_FATAL),
        (R.lw_control(i_solver=abi.IP_SOLVER_NO_SCAT), abi.I_ERR_FATAL),
        (R.lw_control(first_band=3, last_band=12), abi.I_ERR_RANGE),
        (R.lw_control(i_gas_overlap=8), abi.I_ERR_FATAL),
    ]
    for ctl, status in bad:
        with pytest.raises(R.RadianceError) as e:
            R.radiance_calc(ctl, sp, col)
        assert e.value.status == status
    # the library still works afterwards
    out = R.radiance_calc(R.lw_noscat_control(), sp, col)
    assert np.isfinite(out["flux_up"]).all()


def test_band_subrange_matches_oracle(gpu_lib):
    sp, col = synth.config2(16, 60, seed=5)
    ctl = R.sw_control(l_aerosol_mode=True, first_band=2, last_band=4)
    assert_fp64_parity(R.radiance_calc(ctl, sp, col), O.radiance_calc(ctl, sp, col), "bands 2-4: ", mass=col.mass)


def test_kernels_launch_on_device(gpu_lib):
    before = R.launch_count()
    CASES["lw_noscat"](_gpu)
    assert R.launch_count() > before


def test_icrccm27_known_good_output_on_gpu(gpu_lib):
    """The reference's ICRCCM case 27 (HadCM3 LW with continuum, up to 9
    gases per band) through the CUDA path: FP64 against the oracle at
    1e-10, and against the reference's printed heating rates to half a
    unit of their 6th digit; mixed precision within 0.1 W/m2 and
    0.05 K/day."""
    import icrccm27 as K
    ctl, sp, col, kgo = K.load()
    ref = {**O.radiance_calc(ctl, sp, col), "mass": col.mass}
    g64 = {**R.radiance_calc(ctl, sp, col), "mass": col.mass}
    assert_fp64_parity(g64, ref, "icrccm27 fp64: ")
    hr = K.heating_rate(g64, col.mass)[0]
    half_unit = 0.5 * 10.0 ** (np.floor(np.log10(np.abs(kgo))) - 5)
    assert (np.abs(hr - kgo) / half_unit).max() <= 1.0
    gmx = R.radiance_calc(_with(ctl, abi.PRECISION_MIXED), sp, col)
    assert_mixed_tolerance({**gmx, "heating_rate": K.heating_rate(gmx, col.mass)},
                           {**ref, "heating_rate": K.heating_rate(ref, col.mass)}, "icrccm27 mixed: ")


@pytest.mark.parametrize("prec", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_pipelined_host_path_equals_device_path(gpu_lib, prec):
    """socgpu_radiance_calc splits a large batch into column chunks whose
    copies and kernels overlap on several streams; every column must come
    out exactly as from one device-pointer launch."""
    import torch
    from socrates_gb300.device import DeviceCase
    sp, col = synth.config2(5003, 60, seed=31)
    ctl = R.sw_control(l_aerosol_mode=True, precision=prec)
    host = R.radiance_calc(ctl, sp, col)
    dc = DeviceCase(ctl, sp, col)
    dc.run(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for k in ("flux_up", "flux_down", "flux_direct", "heating_rate"):
        np.testing.assert_array_equal(host[k], dc.output(k), err_msg=k)


def _page_locked(a, keep):
    """A page-locked copy of array a (same shape, Fortran order)."""
    import torch
    a = np.asfortranarray(a, dtype=np.int32 if np.issubdtype(np.asarray(a).dtype, np.integer) else np.float64)
    t = torch.empty(a.size, dtype=torch.from_numpy(np.zeros(1, a.dtype)).dtype, pin_memory=True)
    v = t.numpy().reshape(a.shape, order="F")
    v[...] = a
    keep.append(t)
    return v


def _page_locked_call(ctl, sp, col, mc=None):
    """radiance_calc through the C-ABI with every caller array page-locked:
    the pipelined path whose column windows the copy engines move straight
    from the caller's arrays."""
    import ctypes as C
    from dataclasses import replace
    keep = []
    c = copy.copy(col)
    for name in ("p", "t", "p_level", "t_level", "mass", "gas_mix_ratio", "t_ground", "zen_0", "solar_irrad",
                 "rho_alb"):
        if getattr(c, name) is not None:
            setattr(c, name, _page_locked(getattr(c, name), keep))
    if c.aer:
        c.aer = {k: (_page_locked(v, keep) if isinstance(v, np.ndarray) else v) for k, v in c.aer.items()}
    if c.cld:
        c.cld = {k: (_page_locked(v, keep) if isinstance(v, np.ndarray) else v) for k, v in c.cld.items()}
    if mc is not None:
        mc = replace(mc, **{f: _page_locked(getattr(mc, f), keep)
                            for f in ("c_sub", "frac_cloudy", "n_subcol_cld", "subcol_k", "first_subcol_k",
                                      "subcol_reorder") if getattr(mc, f) is not None})
    m = R.Marshal(ctl, sp, c, mc, alloc=lambda *s: _page_locked(np.zeros(s, order="F"), keep))
    lib = R.load_library()
    msg = C.create_string_buffer(512)
    st = lib.socgpu_radiance_calc(*m.args(R.register_spectrum(sp)), msg, 512)
    assert st == abi.I_NORMAL, msg.value.decode()
    return {k: np.array(v) for k, v in m.result().items()}


@pytest.mark.parametrize("prec", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_page_locked_host_path_equals_pageable_path(gpu_lib, prec):
    """Page-locked caller arrays take the pipelined path (each chunk's column
    windows copied straight from them on one stream, the kernel on a second,
    the outputs back on a third); pageable ones are packed into page-locked
    staging first.  Both must give every column bit for bit: the solar
    workload over many chunks, and a McICA batch whose inputs include 4-byte
    integer arrays (n_subcol_cld) and subcolumn fields."""
    sp, col = synth.config2(5003, 60, seed=31)
    ctl = R.sw_control(l_aerosol_mode=True, precision=prec)
    ref = R.radiance_calc(ctl, sp, col)
    got = _page_locked_call(ctl, sp, col)
    for k in ref:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    lw, sw, col3 = synth.config3(3001, 85, seed=5, n_subcol=16)
    synth.add_lw_surface(col3, lw.n_band)
    c_sub, nsc = R.cloud_gen(col3, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_PHILOX)
    mc = R.set_cld_mcica(lw, col3, abi.IP_INFRA_RED, abi.IP_MCICA_SINGLE_SAMPLING, c_sub=c_sub, n_subcol_cld=nsc)
    ctl3 = R.lw_control(i_cloud=abi.IP_CLOUD_MCICA, precision=prec)
    ref3 = R.radiance_calc(ctl3, lw, col3, mc)
    got3 = _page_locked_call(ctl3, lw, col3, mc)
    for k in ref3:
        np.testing.assert_array_equal(got3[k], ref3[k], err_msg="mcica " + k)


def test_full_size_mcica_properties(gpu_lib):
    """The all-sky McICA workload at full size, 65 536 columns x 85 layers x
    16 subcolumns, infra-red.  The GPU generator (Philox) matches the oracle
    bit for bit on 32 sampled columns.  The FP64 path matches the oracle on
    those columns at 1e-10.  Mixed is within 0.1 W/m2 and 0.05 K/day of FP64
    everywhere.  The absorbed flux equals net TOA minus net surface flux."""
    lw, sw, col = synth.config3(65536, 85, seed=3, n_subcol=16)
    synth.add_lw_surface(col, lw.n_band)
    c_sub, nsc = R.cloud_gen(col, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_PHILOX)
    idx = np.sort(np.random.default_rng(1).choice(col.n_profile, 32, replace=False))
    sub = _subset(col, idx)
    o_sub, o_nsc = R.cloud_gen(sub, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_PHILOX, impl=O.cloud_gen_impl)
    np.testing.assert_array_equal(c_sub[idx], o_sub)
    np.testing.assert_array_equal(nsc[idx], o_nsc)
    ctl = R.lw_control(i_cloud=abi.IP_CLOUD_MCICA)
    mc = R.set_cld_mcica(lw, col, abi.IP_INFRA_RED, abi.IP_MCICA_SINGLE_SAMPLING, c_sub=c_sub, n_subcol_cld=nsc)
    g64 = R.radiance_calc(ctl, lw, col, mc)
    gmx = R.radiance_calc(_with(ctl, abi.PRECISION_MIXED), lw, col, mc)
    assert_mixed_tolerance(gmx, g64, "mcica mixed vs fp64: ")
    from dataclasses import replace
    mc_sub = replace(mc, c_sub=np.asfortranarray(c_sub[idx]), n_subcol_cld=np.ascontiguousarray(nsc[idx]),
                     frac_cloudy=np.ascontiguousarray(mc.frac_cloudy[idx]))
    ref = O.radiance_calc(ctl, lw, sub, mc_sub)
    assert_fp64_parity({k: v[idx] for k, v in g64.items()}, ref, "mcica sample: ", mass=col.mass[idx])
    absorbed = g64["flux_div"].sum(axis=1)
    net_toa = g64["flux_down"][:, 0] - g64["flux_up"][:, 0]
    net_sfc = g64["flux_down"][:, -1] - g64["flux_up"][:, -1]
    np.testing.assert_allclose(absorbed, net_toa - net_sfc, rtol=1e-8, atol=1e-6)


# ---------------------------------------------------------------------------
# Two-stream schemes, full-size workloads and edge columns, on both kernel
# families (the `kernel` fixture: scan kernels and the phased kernel).

SCHEMES = {"discrete_ord": abi.IP_DISCRETE_ORD, "pifm85": abi.IP_PIFM85, "2s_test": abi.IP_2S_TEST,
           "hemi_mean": abi.IP_HEMI_MEAN, "eddington": abi.IP_EDDINGTON, "elsasser": abi.IP_ELSASSER,
           "pifm80": abi.IP_PIFM80}


@pytest.mark.parametrize("scheme", sorted(SCHEMES))
@pytest.mark.parametrize("source", ["solar", "infra_red"])
def test_two_stream_schemes_match_oracle(kernel, scheme, source):
    """Every scheme of two_coeff_basic.F90:99-160 (discrete ordinates with
    its own ksi_0, solar_coefficient_basic.F90:171-182), in the solar and the
    infra-red with scattering aerosol: FP64 at 1e-10 and mixed within 0.1
    W/m2 and 0.05 K/day of the oracle."""
    if source == "solar":
        sp, col = synth.config2(16, 60, seed=41)
        ctl = R.sw_control(i_2stream=SCHEMES[scheme], l_aerosol_mode=True)
    else:
        sp, col = synth.config1(16, 60, seed=42)
        synth.add_aerosol(col, sp, 42)
        ctl = R.lw_control(i_2stream=SCHEMES[scheme], l_aerosol_mode=True)
    ref = _ora(ctl, sp, col)
    assert_fp64_parity(_gpu(ctl, sp, col), ref, f"{scheme} {source} fp64: ")
    assert_mixed_tolerance(_gpu(_with(ctl, abi.PRECISION_MIXED), sp, col), ref, f"{scheme} {source} mixed: ")


def test_longwave_clear_sky_full_size(kernel):
    """The plain longwave workload at its stated size, 1000 columns x 60
    layers x 81 g-points, no scattering: every column against the oracle."""
    sp, col = synth.config1(1000, 60, seed=1)
    ctl = R.lw_noscat_control()
    ref = _ora(ctl, sp, col)
    assert_fp64_parity(_gpu(ctl, sp, col), ref, "lw 1000x60 fp64: ")
    assert_mixed_tolerance(_gpu(_with(ctl, abi.PRECISION_MIXED), sp, col), ref, "lw 1000x60 mixed: ")


def _controlled_column(n, L, tau, one_m_om, g, mu0, alb=0.2, seed=43):
    """A solar column whose every cell has the given optical depth, 1-omega
    and asymmetry (arrays of shape (n, L)): no gas absorption, no Rayleigh,
    one aerosol mode carrying all of the extinction."""
    sp, col = synth.config2(n, L, seed=seed)
    col.gas_mix_ratio[...] = 0.0
    nb = sp.n_band
    kt = tau / col.mass
    shape = (n, L, 1, nb)
    col.aer = dict(n_mode=1, mode_mix_ratio=np.asfortranarray(np.ones((n, L, 1))),
                   mode_absorption=np.asfortranarray(np.broadcast_to((kt * one_m_om)[:, :, None, None], shape)),
                   mode_scattering=np.asfortranarray(np.broadcast_to((kt * (1.0 - one_m_om))[:, :, None, None], shape)),
                   mode_asymmetry=np.asfortranarray(np.broadcast_to(g[:, :, None, None], shape)))
    col.zen_0 = np.ascontiguousarray(1.0 / mu0)
    col.rho_alb[...] = alb
    return sp, col


def test_near_conservative_thin_layers(kernel):
    """Thin layers of almost conservative scattering: omega within 1e-7 to
    1e-5 of 1 and lambda tau below 1e-4, where 1 - omega, 1 - gamma and
    1 - T - R lose every digit in a direct FP32 evaluation."""
    n, L = 12, 60
    rng = np.random.default_rng(5)
    tau = 10.0 ** rng.uniform(-4, -2, (n, L))
    one_m_om = 10.0 ** rng.uniform(-7, -5, (n, L))
    g = rng.uniform(0.0, 0.8, (n, L))
    mu0 = rng.uniform(0.1, 1.0, n)
    sp, col = _controlled_column(n, L, tau, one_m_om, g, mu0)
    for rescale in (True, False):
        ctl = R.sw_control(l_aerosol_mode=True, l_rayleigh=False, l_rescale=rescale)
        ref = _ora(ctl, sp, col)
        assert_fp64_parity(_gpu(ctl, sp, col), ref, f"rescale={rescale} fp64: ")
        assert_mixed_tolerance(_gpu(_with(ctl, abi.PRECISION_MIXED), sp, col), ref, f"rescale={rescale} mixed: ")


def _omega_for_lambda(lam, g):
    """1 - omega at which PIFM80 (no rescaling) gives eigenvalue lam for
    asymmetry g: lambda^2 = (2 - 1.5 omega g - 0.5 omega) 2 (1 - omega),
    decreasing in omega; bisection."""
    lo, hi = np.zeros_like(lam), np.ones_like(lam)      # in omega
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        l2 = (2.0 - 1.5 * mid * g - 0.5 * mid) * 2.0 * (1.0 - mid)
        big = l2 > lam * lam
        lo = np.where(big, mid, lo)
        hi = np.where(big, hi, mid)
    return 1.0 - 0.5 * (lo + hi)


def test_solar_singularity_lambda_near_sec0(kernel):
    """Cells whose eigenvalue lambda lies at and around the secant of the
    solar zenith angle, the removable singularity of
    solar_coefficient_basic.F90:124-219.  Two sets of columns, each the same
    column at offsets of lambda from sec_0 of 0, 1e-9, +-1e-6, +-1e-5, +-1e-4,
    +-3e-3 and 1e-2 (relative); optical depth proportional to layer mass.

    * FP64 matches the oracle at 1e-10 where the reference's expressions
      keep that accuracy, |offset| >= 1e-5 (their rounding error grows as
      eps / offset).
    * Exactly on the singularity the reference perturbs lambda by 32 eps,
      which leaves its coefficients with errors of order 1/32 (the oracle
      shows 2 W/m2 at the top of such a column).  The mixed kernel
      interpolates across the singularity instead: it is checked there
      against the oracle's continuous limit, the same column at offset 1e-9,
      and everywhere else against the oracle on its own column."""
    offsets = np.array([0.0, 1e-9, 1e-6, -1e-6, 1e-5, -1e-5, 1e-4, -1e-4, 3e-3, -3e-3, 1e-2])
    no = len(offsets)
    rng = np.random.default_rng(6)
    L, n = 40, 2 * no
    mu0 = np.repeat(rng.uniform(0.55, 1.0, 2), no)
    gs = np.repeat(rng.uniform(0.2, 0.8, 2), no)
    tau_col = np.repeat(rng.uniform(0.5, 3.0, 2), no)
    off = np.tile(offsets, 2)
    sp, col0 = synth.config2(n, L, seed=43)
    tau = col0.mass / col0.mass.sum(axis=1, keepdims=True) * tau_col[:, None]
    g = np.broadcast_to(gs[:, None], (n, L)).copy()
    lam = np.broadcast_to(((1.0 / mu0) * (1.0 + off))[:, None], (n, L))
    sp, col = _controlled_column(n, L, tau, _omega_for_lambda(lam, g), g, mu0)
    ctl = R.sw_control(l_aerosol_mode=True, l_rayleigh=False, l_rescale=False)
    ref = _ora(ctl, sp, col)
    g64 = _gpu(ctl, sp, col)
    sel = np.flatnonzero(np.abs(off) >= 1e-5)
    assert_fp64_parity({k: v[sel] for k, v in g64.items()}, {k: v[sel] for k, v in ref.items()},
                       "singularity fp64: ")
    # the continuous limit for the columns on the singularity
    lim = {k: v.copy() for k, v in ref.items()}
    for c in np.flatnonzero(off == 0.0):
        for k in lim:
            lim[k][c] = ref[k][c + 1]
    assert_mixed_tolerance(_gpu(_with(ctl, abi.PRECISION_MIXED), sp, col), lim, "singularity mixed: ")


def test_full_size_mcica_solar(gpu_lib):
    """The all-sky McICA workload at full size in the solar, 65 536 columns x
    85 layers x 16 subcolumns: FP64 against the oracle on 32 sampled
    columns, mixed against FP64 everywhere, and the energy budget."""
    lw, sw, col = synth.config3(65536, 85, seed=3, n_subcol=16)
    synth.add_sw_surface(col, sw.n_band, 3)
    c_sub, nsc = R.cloud_gen(col, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_PHILOX)
    idx = np.sort(np.random.default_rng(2).choice(col.n_profile, 32, replace=False))
    sub = _subset(col, idx)
    ctl = R.sw_control(i_cloud=abi.IP_CLOUD_MCICA)
    mc = R.set_cld_mcica(sw, col, abi.IP_SOLAR, abi.IP_MCICA_SINGLE_SAMPLING, c_sub=c_sub, n_subcol_cld=nsc)
    g64 = R.radiance_calc(ctl, sw, col, mc)
    gmx = R.radiance_calc(_with(ctl, abi.PRECISION_MIXED), sw, col, mc)
    assert_mixed_tolerance(gmx, g64, "mcica sw mixed vs fp64: ")
    from dataclasses import replace
    mc_sub = replace(mc, c_sub=np.asfortranarray(c_sub[idx]), n_subcol_cld=np.ascontiguousarray(nsc[idx]),
                     frac_cloudy=np.ascontiguousarray(mc.frac_cloudy[idx]))
    ref = O.radiance_calc(ctl, sw, sub, mc_sub)
    assert_fp64_parity({k: v[idx] for k, v in g64.items()}, ref, "mcica sw sample: ", mass=col.mass[idx])
    absorbed = g64["flux_div"].sum(axis=1)
    net_toa = g64["flux_down"][:, 0] - g64["flux_up"][:, 0]
    net_sfc = g64["flux_down"][:, -1] - g64["flux_up"][:, -1]
    np.testing.assert_allclose(absorbed, net_toa - net_sfc, rtol=1e-8, atol=1e-6)


def test_unscaled_direct_beam_under_thick_cloud(gpu_lib):
    """McICA with an overcast, optically thick liquid layer (optical depth
    about 30) and the direct beam reported without delta-scaling
    (i_direct_tau = 0, solar_source.F90:157-176).  There the delta-scaled
    beam is many orders of magnitude above the unscaled one, so the mixed
    kernel has to carry the unscaled beam by itself, not as the scaled beam
    plus a difference.  The direct flux is never negative, and at and below
    the cloud it matches the oracle to 1e-3 relative; FP64 matches at
    1e-10."""
    lw, sw, col = synth.config3(16, 60, seed=13, n_subcol=16)
    synth.add_sw_surface(col, sw.n_band, 13)
    col.zen_0 = np.ascontiguousarray(1.0 / np.random.default_rng(13).uniform(0.5, 1.0, col.n_profile))
    cd = col.cld
    k = 57
    cd["w_cloud"][...] = 0.0
    cd["w_cloud"][:, k] = 1.0
    cd["frac_cloud"][...] = 0.0
    cd["frac_cloud"][:, k, 0] = 1.0
    cd["condensed_mix_ratio"][...] = 0.0
    cd["condensed_mix_ratio"][:, k, 0] = 1.6e-4
    cd["condensed_dim_char"][:, k, 0] = 10.0e-6
    c_sub, nsc = R.cloud_gen(col, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_LCG, impl=O.cloud_gen_impl)
    mc = R.set_cld_mcica(sw, col, abi.IP_SOLAR, abi.IP_MCICA_SINGLE_SAMPLING, c_sub=c_sub, n_subcol_cld=nsc)
    ctl = R.sw_control(i_cloud=abi.IP_CLOUD_MCICA, i_direct_tau=abi.IP_DIRECT_NOSCALING)
    ref = _ora(ctl, sw, col, mc)
    assert_fp64_parity(_gpu(ctl, sw, col, mc), ref, "thick cloud fp64: ")
    gmx = _gpu(_with(ctl, abi.PRECISION_MIXED), sw, col, mc)
    assert gmx["flux_direct"].min() >= 0.0
    below = slice(k + 1, None)
    rel = np.abs(gmx["flux_direct"][:, below] - ref["flux_direct"][:, below]) / ref["flux_direct"][:, below]
    assert ref["flux_direct"][:, below].min() > 0.0
    assert rel.max() <= 1e-3, f"direct flux below the cloud: relative error {rel.max():.3e}"
    assert_mixed_tolerance(gmx, ref, "thick cloud mixed: ")
