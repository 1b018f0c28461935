"""The phased kernel (coefficients of all (k-term, layer) cells in
parallel, then one thread per k-term for the column's recurrences) through
the C-ABI, against the FP64 oracle and against the scan kernels.

Tolerances as in test_parity_gpu: FP64 within 1e-10 of the column's largest
flux; mixed within 0.1 W/m2 and 0.05 K/day.
"""
import numpy as np
import pytest

import oracle as O
from golden_cases import CASES
from socrates_gb300 import abi, synth
from socrates_gb300 import radiance as R
from test_parity_gpu import _gpu, _ora, _subset, _with, assert_fp64_parity, assert_mixed_tolerance

pytestmark = pytest.mark.gpu

CLEAR = sorted(n for n in CASES if not n.startswith("mcica"))


@pytest.fixture
def phased(gpu_lib):
    for prec in (abi.PRECISION_FP64, abi.PRECISION_MIXED):
        for mode in (0, 1):
            assert gpu_lib.socgpu_set_tile_config(prec, mode, 1, 8) == abi.I_NORMAL
    yield
    for prec in (abi.PRECISION_FP64, abi.PRECISION_MIXED):
        for mode in (0, 1):
            gpu_lib.socgpu_set_tile_config(prec, mode, 0, 0)


@pytest.mark.parametrize("name", CLEAR)
def test_phased_fp64_matches_oracle(phased, name):
    assert_fp64_parity(CASES[name](_gpu), CASES[name](_ora), f"{name}: ")


@pytest.mark.parametrize("name", CLEAR)
def test_phased_mixed_within_tolerance(phased, name):
    gpu = CASES[name](lambda c, s, col, mc=None: _gpu(_with(c, abi.PRECISION_MIXED), s, col, mc))
    assert_mixed_tolerance(gpu, CASES[name](_ora), f"{name}: ")


def test_phased_is_deterministic(phased):
    for prec in (abi.PRECISION_FP64, abi.PRECISION_MIXED):
        a = CASES["sw_pifm80"](lambda c, s, col, mc=None: _gpu(_with(c, prec), s, col, mc))
        b = CASES["sw_pifm80"](lambda c, s, col, mc=None: _gpu(_with(c, prec), s, col, mc))
        for k in a:
            np.testing.assert_array_equal(a[k], b[k])


def test_phased_full_size_shortwave(phased):
    """The solar workload at full size (10 000 columns x 100 layers x 48
    g-points): FP64 against the oracle on sampled columns, mixed against
    FP64 everywhere, and the energy budget of every column."""
    sp, col = synth.config2(10000, 100, seed=2)
    ctl = R.sw_control(l_aerosol_mode=True)
    g64 = R.radiance_calc(ctl, sp, col)
    gmx = R.radiance_calc(_with(ctl, abi.PRECISION_MIXED), sp, col)
    idx = np.random.default_rng(0).choice(col.n_profile, 48, replace=False)
    ref = O.radiance_calc(ctl, sp, _subset(col, idx))
    assert_fp64_parity({k: v[idx] for k, v in g64.items()}, ref, "sample: ", mass=col.mass[idx])
    assert_mixed_tolerance(gmx, g64, "mixed vs fp64: ")
    toa_in = col.solar_irrad * sp.solar_flux_band.sum() / col.zen_0
    np.testing.assert_allclose(g64["flux_down"][:, 0], toa_in, rtol=1e-12)
    absorbed = g64["flux_div"].sum(axis=1)
    net_toa = g64["flux_down"][:, 0] - g64["flux_up"][:, 0]
    net_sfc = g64["flux_down"][:, -1] - g64["flux_up"][:, -1]
    np.testing.assert_allclose(absorbed, net_toa - net_sfc, rtol=1e-8, atol=1e-8)


def test_phased_options_it_does_not_cover_run_on_the_scan_kernels(phased):
    """McICA, equivalent extinction and the unscaled direct beam fall back
    to the scan kernels under the phased tile, with the same results."""
    gpu = CASES["mcica_sw_single"](_gpu)
    assert_fp64_parity(gpu, CASES["mcica_sw_single"](_ora), "mcica: ")
    sp, col = synth.config2(8, 60, seed=9)
    ctl = R.sw_control(l_aerosol_mode=True, i_direct_tau=abi.IP_DIRECT_NOSCALING)
    assert_fp64_parity(_gpu(ctl, sp, col), _ora(ctl, sp, col), "unscaled beam: ")


def test_phased_tile_rejected_for_mcica(gpu_lib):
    assert gpu_lib.socgpu_set_tile_config(abi.PRECISION_MIXED, 2, 1, 8) == abi.I_ERR_RANGE
