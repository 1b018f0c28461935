"""Multi-batch launches (socgpu_batch_*) on the GPU.

Every batch of a multi-batch replay must meet the same bars as a single
radiance_calc call: FP64 items within 1e-10 of the oracle (scaled as in the
parity tests), mixed items within 0.1 W/m2 and 0.05 K/day.
"""
from dataclasses import replace

import numpy as np
import pytest

import oracle as O
from golden_cases import CASES
from socrates_gb300 import abi, synth
from socrates_gb300 import radiance as R
from test_parity_gpu import assert_fp64_parity, assert_mixed_tolerance

pytestmark = pytest.mark.gpu

OUT_KEYS = ("flux_up", "flux_down", "flux_direct", "flux_div", "heating_rate")
# layers per lane built for each (precision, lanes): SOCGPU_CHUNKS_* of the library
CHUNKS = {abi.PRECISION_FP64: {16: (4, 8, 16), 32: (4, 5, 8, 16)},
          abi.PRECISION_MIXED: {8: (5, 8, 13, 18), 16: (3, 4, 5, 7, 9, 16), 32: (3, 4, 5, 8, 16)}}


def _capture(name, precision):
    """The (control, spectrum, column, mcica) of a golden case."""
    got = []
    CASES[name](lambda c, s, col, mc=None: got.append((replace(c, precision=precision), s, col, mc)) or {})
    return got[0]


def _outputs(dc):
    return {k: dc.output(k) for k in OUT_KEYS if "out_" + k in dc.tensors}


def _oracle(args):
    c, s, col, mc = args
    return {**O.radiance_calc(c, s, col, mc), "mass": col.mass}


def _check(args, got, tag):
    ref = _oracle(args)
    if args[0].precision == abi.PRECISION_FP64:
        assert_fp64_parity(got, ref, tag, mass=args[2].mass)
    else:
        assert_mixed_tolerance(got, ref, tag)


def test_batch_of_all_cases_matches_oracle(gpu_lib):
    import torch
    from socrates_gb300.batch import Batch
    from socrates_gb300.device import DeviceCase
    args = [(_capture(n, p), f"{n}/{p}") for n in sorted(CASES) for p in (abi.PRECISION_FP64, abi.PRECISION_MIXED)]
    cases = [DeviceCase(a[0], a[1], a[2], a[3]) for a, _ in args]
    b = Batch(cases)
    info = b.info()
    assert info["columns"] == sum(c.n for c in cases)
    before = R.launch_count()
    b.run(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert R.launch_count() - before == info["kernel_classes"]
    for (a, tag), dc in zip(args, cases):
        _check(a, _outputs(dc), tag + ": ")
    b.close()


def test_batch_equals_single_calls_with_the_same_tile(gpu_lib):
    """With the tile fixed per (precision, mode, layers), a batch's results
    equal the single-call path's to rounding: the two kernels run the same
    arithmetic but are compiled in different contexts, so FP32 contractions
    may differ (1e-5 relative for mixed, 1e-12 for FP64)."""
    import torch
    from socrates_gb300.batch import Batch, set_tuned_tile
    from socrates_gb300.device import DeviceCase
    names = ["lw_noscat", "sw_pifm80", "mcica_lw_single", "sw_eddington_137"]
    args = [_capture(n, abi.PRECISION_MIXED) for n in names] + [_capture(n, abi.PRECISION_FP64) for n in names]
    lanes_of_mode = {0: 16, 1: 32, 2: 32}
    for c, s, col, mc in args:
        mode = 2 if c.i_cloud == abi.IP_CLOUD_MCICA else (0 if c.i_scatter_method != abi.IP_SCATTER_FULL else 1)
        lanes = lanes_of_mode[mode]
        chunk = min(ch for ch in CHUNKS[c.precision][lanes] if lanes * ch >= col.n_layer)
        set_tuned_tile(c.precision, mode, col.n_layer, lanes, chunk, 8)
    single = []
    for a in args:
        dc = DeviceCase(*a)
        dc.run(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        single.append(_outputs(dc))
    cases = [DeviceCase(*a) for a in args]
    b = Batch(cases)
    b.run(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for a, dc, ref, n in zip(args, cases, single, names * 2):
        got = _outputs(dc)
        for k in ref:
            scale = np.abs(ref[k]).max() + 1e-300
            err = np.abs(got[k] - ref[k]).max() / scale
            tol = 1e-12 if a[0].precision == abi.PRECISION_FP64 else 1e-5
            assert err <= tol, f"{n} precision {a[0].precision} {k}: {err:.3e}"
    b.close()
    for c, s, col, mc in args:
        mode = 2 if c.i_cloud == abi.IP_CLOUD_MCICA else (0 if c.i_scatter_method != abi.IP_SCATTER_FULL else 1)
        set_tuned_tile(c.precision, mode, col.n_layer, 0, 0, 0)


def _uneven_items(n_batch, seed):
    """Batches of the multi-batch workload's kinds at small sizes: layer
    counts from {38, 60, 85, 137}, LW or SW, clear or all-sky (McICA)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_batch):
        L = int(rng.choice([38, 60, 85, 137]))
        n = int(np.clip(rng.lognormal(np.log(8), 1.0), 1, 48))
        sw = bool(rng.integers(2))
        cloudy = bool(rng.integers(2))
        s = 100 + i
        if cloudy:
            lw_sp, sw_sp, col = synth.config3(n, L, seed=s, n_subcol=16)
            sp = sw_sp if sw else lw_sp
            if sw:
                synth.add_sw_surface(col, sp.n_band, s)
                ctl = R.sw_control(i_cloud=abi.IP_CLOUD_MCICA, precision=abi.PRECISION_MIXED)
            else:
                synth.add_lw_surface(col, sp.n_band)
                ctl = R.lw_control(i_cloud=abi.IP_CLOUD_MCICA, precision=abi.PRECISION_MIXED)
            c_sub, nsc = R.cloud_gen(col, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_PHILOX)
            mc = R.set_cld_mcica(sp, col, ctl.isolir, abi.IP_MCICA_SINGLE_SAMPLING, c_sub=c_sub, n_subcol_cld=nsc)
        elif sw:
            sp, col = synth.config2(n, L, seed=s)
            ctl, mc = R.sw_control(l_aerosol_mode=True, precision=abi.PRECISION_MIXED), None
        else:
            sp, col = synth.config1(n, L, seed=s)
            ctl, mc = R.lw_noscat_control(precision=abi.PRECISION_MIXED), None
        out.append((ctl, sp, col, mc))
    return out


def test_uneven_batches_tuned_match_oracle(gpu_lib):
    import torch
    from socrates_gb300.batch import Batch, tuned_tile
    from socrates_gb300.device import DeviceCase
    items = _uneven_items(24, seed=4)
    cases = [DeviceCase(*a) for a in items]
    b = Batch(cases)
    st = torch.cuda.current_stream().cuda_stream
    b.tune(st, reps=1)
    for c, s, col, mc in items:
        mode = 2 if c.i_cloud == abi.IP_CLOUD_MCICA else (0 if c.i_scatter_method != abi.IP_SCATTER_FULL else 1)
        assert tuned_tile(abi.PRECISION_MIXED, mode, col.n_layer) is not None
    for dc in cases:
        for k in OUT_KEYS:
            if "out_" + k in dc.tensors:
                dc.tensors["out_" + k].fill_(-1.0)
    b.run(st)
    torch.cuda.synchronize()
    for i, (a, dc) in enumerate(zip(items, cases)):
        _check(a, _outputs(dc), f"batch {i} (L={a[2].n_layer}): ")
    b.close()


def test_invalid_item_names_its_index(gpu_lib):
    from socrates_gb300.batch import Batch
    from socrates_gb300.device import DeviceCase
    good = _capture("lw_noscat", abi.PRECISION_MIXED)
    bad = (replace(good[0], i_gas_overlap=8),) + good[1:]      # resort-rebin overlap is not on this path
    with pytest.raises(R.RadianceError) as e:
        Batch([DeviceCase(*good), DeviceCase(*bad)])
    assert e.value.status == abi.I_ERR_FATAL
    assert "batch 1" in str(e.value)
