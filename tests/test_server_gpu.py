"""The continuous-batching request server (socgpu_server_*) on the GPU.

A request's result must be the same alone (one socgpu_radiance_calc call)
and in a mix of concurrent requests: within 0.1 W/m2 and 0.05 K/day for
mixed-precision requests and within 1e-12 relative for FP64 requests.  The
two paths run the same arithmetic in kernels compiled in different contexts,
so only rounding may differ.
"""
import random
import threading
import time

import numpy as np
import pytest

from socrates_gb300 import abi
from socrates_gb300 import radiance as R
from socrates_gb300.workload import Pools, request_specs

pytestmark = pytest.mark.gpu

KEYS = ("flux_up", "flux_down", "flux_direct", "heating_rate")


def _requests(n, seed, median=24.0, precision=abi.PRECISION_MIXED):
    specs = request_specs(n, seed, median=median, sigma=0.8, clip=(1, 256))
    pools = Pools(specs, seed)
    return specs, [pools.request(s, precision) for s in specs]


def _compare(alone, mixed, precision, tag):
    for k in KEYS:
        if k not in alone:
            continue
        a, b = alone[k], mixed[k]
        if precision == abi.PRECISION_FP64:
            err = np.abs(a - b).max() / (np.abs(a).max() + 1e-300)
            assert err <= 1e-12, f"{tag} {k}: {err:.3e} relative"
        else:
            tol = 0.05 if k == "heating_rate" else 0.1
            err = np.abs(a - b).max()
            assert err <= tol, f"{tag} {k}: {err:.4f}"


def test_results_same_alone_and_in_the_mix(gpu_lib):
    from socrates_gb300.server import Server
    specs, reqs = _requests(48, seed=21)
    _, reqs64 = _requests(8, seed=22, precision=abi.PRECISION_FP64)
    reqs = reqs + reqs64
    alone = [R.radiance_calc(*r) for r in reqs]
    marshals = [R.Marshal(*r) for r in reqs]
    srv = Server(device_bytes=256 << 20, streams=4, max_wave_requests=16)
    tickets = [None] * len(reqs)

    def submit(idx):
        rng = random.Random(idx[0])
        for i in idx:
            tickets[i] = srv.submit(marshals[i], reqs[i][1])
            time.sleep(rng.random() * 2e-4)

    order = list(range(len(reqs)))
    threads = [threading.Thread(target=submit, args=(order[j::2],)) for j in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    lat = [srv.wait(t, 60.0) for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs)
    assert st["waves"] >= 1 and st["max_wave_requests"] >= 1
    assert all(q >= 0.0 and l >= q for q, l in lat)
    assert st["column_gpoints"] == sum(r[2].n_profile * r[1].n_gpoint for r in reqs)
    for i, (r, a, m) in enumerate(zip(reqs, alone, marshals)):
        _compare(a, m.result(), r[0].precision, f"request {i}")


def test_admission_bounded_by_device_memory(gpu_lib):
    """With an arena of a few requests, every request still completes, in
    several waves, and the arena's peak use stays within it."""
    from socrates_gb300.server import Server
    specs, reqs = _requests(30, seed=23)
    marshals = [R.Marshal(*r) for r in reqs]
    sizes = []
    for m in marshals:
        sizes.append(sum(a.nbytes for a in m.keep if hasattr(a, "nbytes")) +
                     sum(getattr(m, k).nbytes for k in ("flux_up", "flux_down", "heating_rate")))
    budget = 3 * max(sizes) + (1 << 20)
    srv = Server(device_bytes=budget, streams=3, max_wave_requests=64)
    tickets = [srv.submit(m, r[1]) for m, r in zip(marshals, reqs)]
    for t in tickets:
        srv.wait(t, 60.0)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs)
    assert st["peak_bytes"] <= st["device_bytes"]
    assert st["waves"] > 1
    for r, m in zip(reqs, marshals):
        _compare(R.radiance_calc(*r), m.result(), r[0].precision, "budget")


def test_oversized_request_and_unknown_ticket(gpu_lib):
    from socrates_gb300.server import Server
    _, reqs = _requests(1, seed=24, median=200.0)
    srv = Server(device_bytes=1 << 16, streams=1)
    with pytest.raises(R.RadianceError) as e:
        srv.submit(R.Marshal(*reqs[0]), reqs[0][1])
    assert e.value.status == abi.I_ERR_RANGE
    with pytest.raises(R.RadianceError) as e:
        srv.wait(12345, 0.1)
    assert e.value.status == abi.I_ERR_EXIST
    srv.close()


def test_invalid_request_rejected_at_submit(gpu_lib):
    from dataclasses import replace
    from socrates_gb300.server import Server
    _, reqs = _requests(1, seed=25)
    c, sp, col, mc = reqs[0]
    bad = replace(c, i_gas_overlap=8)
    srv = Server(device_bytes=64 << 20, streams=1)
    with pytest.raises(R.RadianceError) as e:
        srv.submit(R.Marshal(bad, sp, col, mc), sp)
    assert e.value.status == abi.I_ERR_FATAL
    srv.close()


def test_small_requests_overtake_a_large_one(gpu_lib):
    """A large McICA request (8192 columns x 137 layers) and then small
    requests submitted while it runs, all with page-locked host arrays (the
    server's asynchronous path): the small requests go in their own waves,
    on high-priority streams, so at least two waves are on the device at
    once and every small request finishes before the large one; each result
    is still the same as alone."""
    from socrates_gb300.server import Server
    from socrates_gb300.workload import PinnedArena, RequestSpec, pin_outputs
    big_spec = RequestSpec("sw_cloudy", 137, 8192, 0.0)
    small_specs = request_specs(8, 32, median=16.0, sigma=0.8, clip=(1, 64))
    pools = Pools([big_spec] + small_specs, 31)
    arena = PinnedArena(1 << 30)
    reqs = [pools.request(q, abi.PRECISION_MIXED, arena.take) for q in [big_spec] + small_specs]
    marshals = [pin_outputs(R.Marshal(*r), arena.take) for r in reqs]
    srv = Server(device_bytes=2 << 30, streams=4, max_wave_requests=16)
    for m, r in zip(marshals[1:], reqs[1:]):          # every kernel class once, before timing
        srv.wait(srv.submit(m, r[1]), 60.0)
    t0 = time.perf_counter()
    t_big = srv.submit(marshals[0], reqs[0][1])
    ts = []
    for m, r in zip(marshals[1:], reqs[1:]):
        ts.append((srv.submit(m, r[1]), time.perf_counter() - t0))
        time.sleep(2e-4)
    done_small = []
    for t, sub in ts:
        _, lat = srv.wait(t, 60.0)
        done_small.append(sub * 1e3 + lat)
    _, lat_big = srv.wait(t_big, 60.0)
    st = srv.stats()
    srv.close()
    colg = [r[2].n_profile * r[1].n_gpoint for r in reqs]
    diag = f"small done at {[round(x, 3) for x in done_small]} ms, large at {lat_big:.3f} ms, stats {st}, colg {colg}"
    assert colg[0] > max(colg[1:]), diag
    assert st["max_waves_in_flight"] >= 2, diag
    assert st["small_waves"] >= 1, diag
    assert max(done_small) < lat_big, diag
    for r, m in zip(reqs, marshals):
        _compare(R.radiance_calc(*r), m.result(), r[0].precision, "overtake")
