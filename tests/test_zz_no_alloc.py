"""socgpu_cloud_gen_device_noalloc: the allocation-free cloud generator.

It must give the same subcolumns, bit for bit, as socgpu_cloud_gen_device on
the same device inputs, on consecutive calls that share its fixed scratch.
This file is collected last so that the GPU test also runs after every other
test in the session has used the library.
"""
import ctypes as C

import numpy as np
import pytest

from socrates_gb300 import abi, build, synth


def _lib():
    from socrates_gb300 import radiance
    build.build()
    return radiance.load_library()


def _gen_inputs(col, ict=0):
    """cloud_gen inputs of a column batch as Fortran-ordered numpy arrays."""
    cd = col.cld
    n, L = col.n_profile, col.n_layer
    zero = np.zeros((n, L - ict), order="F")
    return dict(
        seeds=np.ascontiguousarray(cd["rand_seed"], dtype=np.int32),
        rlc_cf=np.asfortranarray(cd["dp_corr_cloud"][:, ict:]),
        rlc_cw=np.asfortranarray(cd["dp_corr_cond"][:, ict:]),
        sigma=zero, avg_cf=np.asfortranarray(cd["w_cloud"][:, ict:]), c_cloud=zero, c_ratio=zero,
        zf=np.asfortranarray(col.p), xcw=np.zeros((2, 2), order="F"))


class _Device:
    """Inputs and outputs of one cloud_gen call in device memory."""

    def __init__(self, inp, n, ndc, n_subcol):
        import torch
        self.keep = {k: torch.from_numpy(np.ravel(v, order="F").copy()).cuda() for k, v in inp.items()}
        self.nsc = torch.zeros(n, dtype=torch.int32, device="cuda")
        self.c_sub = torch.full((n * ndc * n_subcol,), -1.0, dtype=torch.float64, device="cuda")

    def ptr(self, k):
        return C.c_void_p(self.keep[k].data_ptr())

    def outputs(self, n, ndc, n_subcol):
        c = self.c_sub.cpu().numpy().reshape((n, ndc, n_subcol), order="F")
        return c, self.nsc.cpu().numpy()


def _call(fn, dev, n, L, n_subcol, ioverlap, rng, stream):
    msg = C.create_string_buffer(512)
    st = fn(L, 1, L, n, 1, n, n_subcol, 2, 2, 0, ioverlap, dev.ptr("seeds"), dev.ptr("rlc_cf"), dev.ptr("rlc_cw"),
            dev.ptr("sigma"), dev.ptr("avg_cf"), dev.ptr("c_cloud"), dev.ptr("c_ratio"), dev.ptr("zf"),
            dev.ptr("xcw"), C.c_void_p(dev.nsc.data_ptr()), C.c_void_p(dev.c_sub.data_ptr()), rng,
            C.c_void_p(stream), msg, 512)
    assert st == abi.I_NORMAL, msg.value.decode()


def _two_batches(n, L, n_subcol):
    """Two batches whose cloudy layer ranges differ: the second has cloud only
    in layers 40..55 and, above them, cloud fractions of 1e-17 (below the
    generator's cut, so outside its layer range).  A range left over from the
    first batch would take those layers in and shift the LCG stream."""
    _, _, c1 = synth.config3(n, L, seed=11, n_subcol=n_subcol)
    _, _, c2 = synth.config3(n, L, seed=12, n_subcol=n_subcol)
    w = c2.cld["w_cloud"].copy()
    w[:, :40] = 0.0
    w[:, 56:] = 0.0
    w[:, 10:40] = 1e-17
    w[:, 40:56] = np.maximum(w[:, 40:56], 0.3)
    c2.cld["w_cloud"] = w
    return c1, c2


@pytest.mark.gpu
@pytest.mark.parametrize("rng", [abi.RNG_LCG, abi.RNG_PHILOX])
@pytest.mark.parametrize("ioverlap", [abi.IP_MAX_RAND, abi.IP_EXPONENTIAL_RAND])
def test_noalloc_matches_cloud_gen_device_on_consecutive_calls(ioverlap, rng):
    import torch
    lib = _lib()
    n, L, n_subcol = 384, 85, 16
    c1, c2 = _two_batches(n, L, n_subcol)
    stream = torch.cuda.current_stream().cuda_stream
    ref, new = [], []
    for col in (c1, c2):
        d = _Device(_gen_inputs(col), n, L, n_subcol)
        _call(lib.socgpu_cloud_gen_device, d, n, L, n_subcol, ioverlap, rng, stream)
        torch.cuda.synchronize()
        ref.append(d.outputs(n, L, n_subcol))
    # two calls in a row on one stream, no synchronisation between them
    devs = [_Device(_gen_inputs(col), n, L, n_subcol) for col in (c1, c2)]
    for d in devs:
        _call(lib.socgpu_cloud_gen_device_noalloc, d, n, L, n_subcol, ioverlap, rng, stream)
    torch.cuda.synchronize()
    new = [d.outputs(n, L, n_subcol) for d in devs]
    for (rc, rn), (nc, nn) in zip(ref, new):
        np.testing.assert_array_equal(nn, rn)
        np.testing.assert_array_equal(nc, rc)
        assert rn.max() > 0


@pytest.mark.gpu
def test_second_batch_is_sensitive_to_the_layer_range():
    """The second batch of the consecutive-call test tells a stale layer range
    apart: with its 1e-17 layers raised above the cut (the range then starts
    at layer 10) the LCG subcolumns change."""
    import torch
    lib = _lib()
    n, L, n_subcol = 384, 85, 16
    _, c2 = _two_batches(n, L, n_subcol)
    stream = torch.cuda.current_stream().cuda_stream
    out = []
    for tiny in (1e-17, 1e-10):
        inp = _gen_inputs(c2)
        inp["avg_cf"] = inp["avg_cf"].copy(order="F")
        inp["avg_cf"][:, 10:40] = tiny
        d = _Device(inp, n, L, n_subcol)
        _call(lib.socgpu_cloud_gen_device_noalloc, d, n, L, n_subcol, abi.IP_EXPONENTIAL_RAND, abi.RNG_LCG, stream)
        torch.cuda.synchronize()
        out.append(d.outputs(n, L, n_subcol))
    assert not np.array_equal(out[0][0], out[1][0])


def test_noalloc_rejects_more_layers_than_its_scratch_holds():
    """Beyond SOCGPU_NOALLOC_MAX_CLOUD_LAYERS the call fails with a range
    error and a message before touching any pointer or the device."""
    lib = _lib()
    L = abi.NOALLOC_MAX_CLOUD_LAYERS + 1
    msg = C.create_string_buffer(512)
    before = lib.socgpu_kernel_launch_count()
    null = C.c_void_p(0)
    st = lib.socgpu_cloud_gen_device_noalloc(L, 1, L, 8, 1, 8, 4, 2, 2, 0, abi.IP_EXPONENTIAL_RAND, *([null] * 9),
                                             null, null, abi.RNG_LCG, null, msg, 512)
    assert st == abi.I_ERR_RANGE
    assert b"allocation-free limit" in msg.value
    assert lib.socgpu_kernel_launch_count() == before
