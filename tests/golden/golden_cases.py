"""Small seeded cases shared by the golden fixtures, the oracle tests and the
GPU parity tests.  Each case builds its inputs with socrates_gb300.synth and
runs a radiance_calc implementation passed in as `run(control, spectrum,
column, mcica=None)`."""
import numpy as np

from socrates_gb300 import abi, synth
from socrates_gb300 import radiance as R


def lw_noscat(run, precision=abi.PRECISION_FP64):
    sp, col = synth.config1(24, 60, seed=1)
    return run(R.lw_noscat_control(precision=precision), sp, col)


def lw_noscat_linear(run, precision=abi.PRECISION_FP64):
    sp, col = synth.config1(16, 38, seed=11)
    return run(R.lw_noscat_control(l_ir_source_quad=False, precision=precision), sp, col)


def lw_scatter_aerosol(run, precision=abi.PRECISION_FP64):
    sp, col = synth.config1(16, 85, seed=12)
    synth.add_aerosol(col, sp, 12)
    return run(R.lw_control(l_aerosol_mode=True, precision=precision), sp, col)


def sw_pifm80(run, precision=abi.PRECISION_FP64):
    sp, col = synth.config2(24, 100, seed=2)
    return run(R.sw_control(l_aerosol_mode=True, precision=precision), sp, col)


def sw_eddington_137(run, precision=abi.PRECISION_FP64):
    sp, col = synth.config2(12, 137, seed=21)
    return run(R.sw_control(i_2stream=abi.IP_EDDINGTON, l_aerosol_mode=True, precision=precision), sp, col)


def _mcica(run, isolir, precision, sampling):
    lw, sw, col = synth.config3(16, 85, seed=3, n_subcol=16)
    sp = sw if isolir == abi.IP_SOLAR else lw
    if isolir == abi.IP_SOLAR:
        synth.add_sw_surface(col, sp.n_band, 3)
        ctl = R.sw_control(i_cloud=abi.IP_CLOUD_MCICA, precision=precision)
    else:
        synth.add_lw_surface(col, sp.n_band)
        ctl = R.lw_control(i_cloud=abi.IP_CLOUD_MCICA, precision=precision)
    from oracle import cloud_gen_impl
    c_sub, nsc = R.cloud_gen(col, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_LCG, impl=cloud_gen_impl)
    mc = R.set_cld_mcica(sp, col, isolir, sampling, c_sub=c_sub, n_subcol_cld=nsc)
    return run(ctl, sp, col, mc)


def mcica_lw_single(run, precision=abi.PRECISION_FP64):
    return _mcica(run, abi.IP_INFRA_RED, precision, abi.IP_MCICA_SINGLE_SAMPLING)


def mcica_sw_single(run, precision=abi.PRECISION_FP64):
    return _mcica(run, abi.IP_SOLAR, precision, abi.IP_MCICA_SINGLE_SAMPLING)


def mcica_sw_full(run, precision=abi.PRECISION_FP64):
    return _mcica(run, abi.IP_SOLAR, precision, abi.IP_MCICA_FULL_SAMPLING)


CASES = {f.__name__: f for f in (lw_noscat, lw_noscat_linear, lw_scatter_aerosol, sw_pifm80, sw_eddington_137,
                                 mcica_lw_single, mcica_sw_single, mcica_sw_full)}
