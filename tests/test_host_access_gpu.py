"""Page-locked caller arrays through socgpu_radiance_calc: the copy pipeline
(SOCGPU_HOST_ACCESS=copy) and the kernel reading and writing them in place
through their mapped addresses (SOCGPU_HOST_ACCESS=direct) give the same
fluxes bit for bit."""
import ctypes as C
import os

import numpy as np
import pytest

from socrates_gb300 import abi, synth
from socrates_gb300 import radiance as R

pytestmark = pytest.mark.gpu


def _pinned(keep):
    import torch

    def alloc(*shape):
        t = torch.zeros(int(np.prod(shape)), dtype=torch.float64).pin_memory()
        keep.append(t)
        return t.numpy().reshape(shape, order="F")
    return alloc


def _pin_column(col, alloc):
    for name in ("p", "t", "p_level", "t_level", "mass", "gas_mix_ratio", "density", "zen_0", "solar_irrad",
                 "rho_alb", "t_ground"):
        a = getattr(col, name)
        if isinstance(a, np.ndarray):
            b = alloc(*a.shape)
            b[...] = a
            setattr(col, name, b)
    if col.aer:
        for k, a in list(col.aer.items()):
            if isinstance(a, np.ndarray) and a.dtype == np.float64:
                b = alloc(*a.shape)
                b[...] = a
                col.aer[k] = b


def _run(ctl, sp, col, mode, alloc):
    os.environ["SOCGPU_HOST_ACCESS"] = mode
    try:
        lib = R.load_library()
        h = R.register_spectrum(sp)
        m = R.Marshal(ctl, sp, col, alloc=alloc)
        msg = C.create_string_buffer(512)
        st = lib.socgpu_radiance_calc(*m.args(h), msg, 512)
        assert st == abi.I_NORMAL, msg.value.decode()
        return {k: np.array(v) for k, v in m.result().items()}
    finally:
        os.environ.pop("SOCGPU_HOST_ACCESS", None)


@pytest.mark.parametrize("prec", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_direct_host_access_equals_copies(gpu_lib, prec):
    keep = []
    alloc = _pinned(keep)
    sp, col = synth.config2(4001, 60, seed=71)
    _pin_column(col, alloc)
    ctl = R.sw_control(l_aerosol_mode=True, precision=prec)
    a = _run(ctl, sp, col, "copy", alloc)
    b = _run(ctl, sp, col, "direct", alloc)
    for k in ("flux_up", "flux_down", "flux_direct", "heating_rate"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert np.abs(a["flux_down"]).max() > 100.0
