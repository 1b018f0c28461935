"""Benchmark of the two-stream flux path on one GB300 (or N replicas).

Workload: shortwave PIFM80 two-stream with delta-Eddington rescaling,
Rayleigh and one aerosol mode, direct + diffuse solve: 10 000 columns x
100 layers x 48 g-points (6 bands x 8 k-terms), seeded synthetic inputs
(socrates_gb300.synth.config2).  A step is one radiance_calc pass over
the batch.  The headline path is the mixed FP32/FP64 kernel; the plain
FP64 device path, the mixed-vs-FP64 error and the CPU baseline are
reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
    python bench.py --workload batched [--batches 4096]

`--workload batched` runs the multi-batch workload instead: 4096 column
batches of log-normal width (median 256), layer counts from {38, 60, 85,
137}, LW or SW, clear or all-sky McICA (socrates_gb300.workload), replayed
as one CUDA graph of autotuned persistent launches.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "column·g-pts/s mixed vs FP64 at ≤0.1 W/m² flux error; serve p50/p99 ms"
UNIT = "column·g-points/s"
N_COL, N_LAYER, SEED = 10000, 100, 2
CONFIG = {"workload": "SW PIFM80 delta-Eddington direct+diffuse, Rayleigh + modal aerosol, "
                      "10000 columns x 100 layers, 6 bands x 8 k-terms (48 g-points)",
          "columns": N_COL, "layers": N_LAYER, "g_points": 48, "precision": "mixed FP32/FP64",
          "l2": "256 MiB L2 flush between timed steps; inputs (about 200 MB) exceed the 129 MB L2"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default 200; 20 for --workload batched)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="socgpu", choices=["socgpu", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=N_COL, help="columns of the CPU baseline sample")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU work of the baseline sample")
    ap.add_argument("--workload", default="sw", choices=["sw", "batched", "serve", "ga9"])
    ap.add_argument("--rates", default="200,1000,5000", help="arrival rates (requests/s) of the serving workload")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="arrival window per rate")
    ap.add_argument("--batches", type=int, default=4096, help="column batches of the batched workload")
    ap.add_argument("--batched-steps", type=int, default=10, help="timed graph replays of the batched workload")
    ap.add_argument("--no-extras", action="store_true",
                    help="the default run without the multi-batch and serving figures")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons (read only)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0:   # first sample before the timed region
                time.sleep(0.02)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def profile_figures():
    """Per-launch DRAM bytes and warp instructions of the mixed flux kernel,
    read from the committed ncu summary (lines ``name: value``)."""
    p = ROOT / "profiles" / "flux_kernel_sw_mixed_10000x100x48.md"
    out = {}
    if p.exists():
        for line in p.read_text().splitlines():
            key, _, val = line.strip().partition(":")
            if key in ("dram_bytes_per_launch", "warp_instructions_per_launch") and val.strip().isdigit():
                out[key] = int(val.strip())
    return out


def cpu_baseline(n_sample: int, min_seconds: float = 10.0):
    """The FP64 oracle (a C restatement of the reference) on all host cores
    over a bounded sample of the workload: n_sample columns, repeated until
    about min_seconds of CPU work have run."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from socrates_gb300 import radiance as R
    from socrates_gb300.synth import config2
    threads = os.cpu_count() or 1
    sp_s, col_s = config2(n_sample, N_LAYER, SEED)
    ctl = R.sw_control(l_aerosol_mode=True)
    O.radiance_calc(ctl, sp_s, config2(threads, N_LAYER, SEED)[1], threads=threads)   # warm-up
    reps, t0 = 0, time.perf_counter()
    while True:
        O.radiance_calc(ctl, sp_s, col_s, threads=threads)
        reps += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds or reps >= 1000:
            break
    return {"value": reps * n_sample * sp_s.n_gpoint / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "seconds": dt, "sample": f"{reps} passes over {n_sample} of the workload's {N_COL} columns (all 100 layers, "
                                     f"48 g-points), FP64 C restatement with OpenMP over column segments"}


def dist_setup(n: int):
    rank, world = 0, 1
    if n > 1 or "RANK" in os.environ:
        import torch.distributed as dist
        rank = int(os.environ.get("RANK", 0))
        world = int(os.environ.get("WORLD_SIZE", n))
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device="cuda", dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    """CPU reference arm: the oracle port on all host cores, same metric."""
    rank = int(os.environ.get("RANK", 0))
    if rank != 0:
        return
    from socrates_gb300.synth import config2
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from socrates_gb300 import radiance as R
    threads = os.cpu_count() or 1
    n = args.cpu_sample
    sp, col = config2(n, N_LAYER, SEED)
    ctl = R.sw_control(l_aerosol_mode=True)
    for _ in range(args.warmup):
        O.radiance_calc(ctl, sp, col, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.radiance_calc(ctl, sp, col, threads=threads)
    dt = (time.perf_counter() - t0) / args.steps
    value = n * sp.n_gpoint / dt
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox, shapes of the workload)",
            "config": {**CONFIG, "precision": "FP64", "columns": n},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{n} of {N_COL} columns per step, all 100 layers and 48 g-points, FP64 C "
                                       f"restatement of the reference (no Fortran compiler on the box)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batched_figures(args, rank: int = 0, world: int = 1) -> dict:
    """The multi-batch workload: 4096 uneven column batches replayed as one
    CUDA graph of autotuned launches, the same batches one call each (mixed
    and FP64), and the mixed-vs-FP64 error over all of them."""
    import torch
    from socrates_gb300 import abi
    from socrates_gb300 import build as B
    from socrates_gb300 import radiance as R
    from socrates_gb300.batch import Batch
    from socrates_gb300.device import DeviceCase
    from socrates_gb300.workload import Pools, request_specs
    B.build()
    dev = torch.cuda.current_device()
    seed = 4 + rank
    t_setup = time.perf_counter()
    specs = request_specs(args.batches, seed)
    pools = Pools(specs, seed)
    cases = [DeviceCase(*pools.request(s, abi.PRECISION_MIXED), keep_host=False) for s in specs]
    t_setup = time.perf_counter() - t_setup
    stream = torch.cuda.current_stream()
    batch = Batch(cases)
    t_tune = time.perf_counter()
    batch.tune(stream.cuda_stream, reps=2)
    torch.cuda.synchronize()
    t_tune = time.perf_counter() - t_tune
    info = batch.info()
    colg = info["column_gpoints"]
    in_bytes = sum(c.input_bytes for c in cases)
    for _ in range(max(3, args.warmup)):
        batch.run(stream.cuda_stream)
    torch.cuda.synchronize()
    barrier(world)
    steps = max(1, args.batched_steps)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    l0 = R.launch_count()
    with ClockSampler(dev) as clk:
        for e0, e1 in evs:
            e0.record(stream)
            batch.run(stream.cuda_stream)
            e1.record(stream)
        torch.cuda.synchronize()
    launches = R.launch_count() - l0
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs) / steps, world)
    value = world * colg / (ms * 1e-3)

    # the same requests one call each, without batching, mixed and FP64
    def per_request(cs, reps):
        for c in cs:
            c.run(stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            for c in cs:
                c.run(stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps
    ms_single = per_request(cases, 2)
    cases64 = [c.clone(abi.PRECISION_FP64) for c in cases]
    ms_64 = per_request(cases64, 1)
    batch.run(stream.cuda_stream)
    torch.cuda.synchronize()
    err_flux = err_hr = 0.0
    for c, c64 in zip(cases, cases64):
        for k in ("flux_up", "flux_down", "flux_direct"):
            if "out_" + k in c.tensors:
                err_flux = max(err_flux, float((c.tensors["out_" + k] - c64.tensors["out_" + k]).abs().max()))
        err_hr = max(err_hr, float((c.tensors["out_heating_rate"] - c64.tensors["out_heating_rate"]).abs().max()))
    kinds = {}
    for s in specs:
        kinds[s.kind] = kinds.get(s.kind, 0) + 1
    out = {"value": value, "unit": UNIT, "ms_per_step": ms, "steps": steps,
           "config": {"workload": f"{args.batches} uneven column batches in one CUDA-graph replay: columns "
                                  "log-normal (median 256, sigma 1, clip 1-8192), layers from {38,60,85,137}, "
                                  "LW 81 / SW 48 g-points, clear or McICA all-sky (16 subcolumns), mixed precision",
                      "batches": args.batches, "columns": info["columns"], "column_gpoints": colg,
                      "kinds": kinds, "kernel_classes": info["kernel_classes"],
                      "l2": f"inputs {in_bytes / 1e9:.1f} GB, far above the 129 MB L2; no flush needed"},
           "per_request_mixed": {"value": world * colg / (ms_single * 1e-3), "ms_per_step": ms_single,
                                 "note": "the same requests, one socgpu_radiance_calc_device call each"},
           "fp64_per_request": {"value": world * colg / (ms_64 * 1e-3), "ms_per_step": ms_64,
                                "note": "the same requests in FP64, one call each (the plain FP64 GPU path)"},
           "speedup_batched_mixed_over_fp64": ms_64 / ms,
           "accuracy_vs_fp64": {"max_flux_err_wm2": err_flux, "max_heating_rate_err_kday": err_hr},
           "setup_s": t_setup, "tune_s": t_tune, "gpu_launches": int(launches), "clocks": clk.summary()}
    del batch, cases, cases64
    torch.cuda.empty_cache()
    return out


def run_batched(args):
    """The multi-batch workload as its own bench line."""
    rank, world = dist_setup(args.gpus)
    f = batched_figures(args, rank, world)
    if rank == 0:
        line = {"metric": METRIC, "value": f["value"], "unit": UNIT, "n_gpus": world, "steps": f["steps"],
                "warmup": max(3, args.warmup), "ms_per_step": f["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic (seeded windows of per-kind pools)", "config": f["config"],
                **{k: f[k] for k in ("per_request_mixed", "fp64_per_request", "speedup_batched_mixed_over_fp64",
                                     "accuracy_vs_fp64", "setup_s", "tune_s", "gpu_launches", "clocks")}}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def serve_figures(args, rank: int = 0) -> dict:
    """The serving workload: Poisson arrivals of requests drawn like the
    multi-batch workload, served by the continuous-batching server; p50/p99
    latency and throughput per arrival rate, beside the plain FP64
    per-request GPU path on the same arrival trace and the CPU port."""
    import ctypes
    import numpy as np
    import torch
    from dataclasses import replace
    from socrates_gb300 import abi
    from socrates_gb300 import build as B
    from socrates_gb300 import radiance as R
    from socrates_gb300.server import Server
    from socrates_gb300.workload import PinnedArena, Pools, pin_outputs, request_specs
    B.build()
    rates = [float(r) for r in args.rates.split(",")]
    seed = 5 + rank
    # 128 request slots: page-locked inputs and outputs drawn like the
    # multi-batch workload; request i of a trace uses slot i mod 128, once
    # the slot's previous request has finished
    n_slot = 128
    specs = request_specs(n_slot, seed)
    pools = Pools(specs, seed)

    def need(s):
        return s.n_profile * (s.n_layer + 1) * 8 * 48 + (1 << 16)
    arena = PinnedArena(sum(need(s) for s in specs) + (64 << 20))
    slots = []
    for s in specs:
        ctl, sp, col, mc = pools.request(s, abi.PRECISION_MIXED, arena.take)
        m = pin_outputs(R.Marshal(ctl, sp, col, mc), arena.take)
        slots.append((m, sp, (ctl, sp, col, mc)))
        R.register_spectrum(sp)
    srv = Server(device_bytes=0, streams=4, max_wave_requests=256)
    for i in range(n_slot):                      # warm-up: every kernel class once
        srv.wait(srv.submit(slots[i][0], slots[i][1]))
    results = []
    for rate in rates:
        n = int(rate * args.serve_seconds)
        rng = np.random.default_rng(int(rate))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
        tickets = [None] * n
        lat = [0.0] * n
        queue = [0.0] * n
        done = [0]
        cv = threading.Condition()

        def waiter():
            for i in range(n):
                with cv:
                    cv.wait_for(lambda: tickets[i] is not None)
                queue[i], lat[i] = srv.wait(tickets[i])
                with cv:
                    done[0] = i + 1
                    cv.notify_all()
        th = threading.Thread(target=waiter)
        th.start()
        s0 = srv.stats()
        t0 = time.perf_counter()
        late = 0
        for i in range(n):
            if i >= n_slot:
                with cv:
                    cv.wait_for(lambda: done[0] > i - n_slot)
            while time.perf_counter() - t0 < arrivals[i]:
                pass
            late += (time.perf_counter() - t0 - arrivals[i]) > 1e-3
            m, sp, _ = slots[i % n_slot]
            t = srv.submit(m, sp)
            with cv:
                tickets[i] = t
                cv.notify_all()
        th.join()
        t_end = time.perf_counter()
        s1 = srv.stats()
        colg = s1["column_gpoints"] - s0["column_gpoints"]
        results.append({"rate_rps": rate, "requests": n, "p50_ms": float(np.percentile(lat, 50)),
                        "p99_ms": float(np.percentile(lat, 99)), "queue_p99_ms": float(np.percentile(queue, 99)),
                        "column_gpoints_per_s": colg / max(t_end - t0, 1e-9),
                        "offered_column_gpoints_per_s": colg / max(float(arrivals[-1]), 1e-9),
                        "submits_late_over_1ms": int(late), "waves": s1["waves"] - s0["waves"],
                        "max_wave_requests": s1["max_wave_requests"], "peak_device_bytes": s1["peak_bytes"]})
    srv.close()
    # the plain FP64 per-request GPU path on the same arrival trace (first
    # 200 requests of each rate): one synchronous socgpu_radiance_calc per
    # request, in arrival order, latency from arrival to return
    lib = R.load_library()
    fp64 = []
    m64 = []
    for m, sp, (ctl, sp_, col, mc) in slots:
        m64.append((R.Marshal(replace(ctl, precision=abi.PRECISION_FP64), sp, col, mc), sp))
    msg = ctypes.create_string_buffer(256)
    for rate in rates:
        n = min(200, int(rate * args.serve_seconds))
        rng = np.random.default_rng(int(rate))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
        lat = []
        colg = 0
        t0 = time.perf_counter()
        for i in range(n):
            m, sp = m64[i % n_slot]
            while time.perf_counter() - t0 < arrivals[i]:
                pass
            st = lib.socgpu_radiance_calc(*m.args(R.register_spectrum(sp)), msg, 256)
            if st != 0:
                raise SystemExit(f"FP64 request failed: {msg.value.decode()}")
            lat.append((time.perf_counter() - t0 - arrivals[i]) * 1e3)
            colg += m.n * sp.n_gpoint
        fp64.append({"rate_rps": rate, "requests": n, "p50_ms": float(np.percentile(lat, 50)),
                     "p99_ms": float(np.percentile(lat, 99)),
                     "column_gpoints_per_s": colg / (time.perf_counter() - t0)})
    # the CPU port on a sample of the same requests (about --cpu-seconds)
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    colg, k = 0, 0
    while time.perf_counter() - t0 < args.cpu_seconds and k < n_slot:
        ctl, sp, col, mc = slots[k][2]
        O.radiance_calc(replace(ctl, precision=abi.PRECISION_FP64), sp, col, mc, threads=threads)
        colg += col.n_profile * sp.n_gpoint
        k += 1
    cpu = {"value": colg / (time.perf_counter() - t0), "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{k} requests of the trace, one FP64 oracle call each, OpenMP over column segments"}
    return {"results": results, "fp64_per_request": fp64, "cpu_baseline": cpu, "rates_rps": rates,
            "window_s": args.serve_seconds, "request_slots": n_slot,
            "config": {"workload": "serving: Poisson arrivals, requests drawn like the multi-batch workload "
                                   "(log-normal columns, median 256; layers {38,60,85,137}; LW/SW; clear or "
                                   "McICA), page-locked host arrays, continuous batching over 4 streams "
                                   "(2 high-priority for small requests)",
                       "rates_rps": rates, "window_s": args.serve_seconds, "request_slots": n_slot}}


def run_serve(args):
    """The serving workload as its own bench line."""
    rank, world = dist_setup(args.gpus)
    f = serve_figures(args, rank)
    if rank == 0:
        best = max(f["results"], key=lambda r: r["column_gpoints_per_s"])
        line = {"metric": METRIC, "value": best["column_gpoints_per_s"], "unit": UNIT, "n_gpus": world,
                "steps": len(f["rates_rps"]), "warmup": 1, "ms_per_step": None, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic (seeded windows of per-kind pools)", "config": f["config"],
                "serve": f["results"], "fp64_per_request": f["fp64_per_request"], "cpu_baseline": f["cpu_baseline"]}
        print(json.dumps(line), flush=True)


def run_ga9(args):
    """The operational spectral files: the GA9 long-wave and short-wave files
    (lookup-table k, Wen-Yi CO2 terms, equivalent-extinction overlap,
    continuum) on 10000 columns of 100 layers, mixed and FP64 device paths;
    the inputs are resident and a 256 MiB L2 flush runs between steps."""
    import numpy as np
    import torch
    rank, world = dist_setup(args.gpus)
    from pathlib import Path
    from dataclasses import replace
    from socrates_gb300 import abi
    from socrates_gb300 import build as B
    from socrates_gb300 import radiance as R
    from socrates_gb300.device import DeviceCase
    from socrates_gb300.spectrum import Spectrum
    from socrates_gb300.synth import operational_case
    if rank == 0:
        B.build()
    barrier(world)
    fixture = Path(__file__).resolve().parent / "tests" / "golden" / "runes_ga9.npz"
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    lines = {}
    for solar in (False, True):
        sp = Spectrum.load_npz(fixture, prefix="sw_" if solar else "lw_")
        col = operational_case(sp, N_COL, N_LAYER, seed=SEED + rank, solar=solar)
        common = dict(l_continuum=True, i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL, l_flux_div=False)
        ctl = R.sw_control(l_rayleigh=True, **common) if solar else R.lw_control(**common)
        res = {}
        for prec, steps in ((abi.PRECISION_MIXED, args.steps), (abi.PRECISION_FP64, max(3, args.steps // 20))):
            case = DeviceCase(replace(ctl, precision=prec), sp, col)
            for _ in range(args.warmup):
                case.run(stream.cuda_stream)
            torch.cuda.synchronize()
            ms = []
            for _ in range(steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                case.run(stream.cuda_stream)
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            t = max_over_ranks(float(np.mean(ms)) / 1e3, world)
            res[prec] = (t, {k: case.output(k).copy() for k in ("flux_up", "flux_down", "heating_rate")})
        (t_mx, o_mx), (t_64, o_64) = res[abi.PRECISION_MIXED], res[abi.PRECISION_FP64]
        # the solves under k_eqv_scl: the k-terms of each band's first
        # absorber (one grey solve in a band without absorbers)
        g = sum(int(sp.i_band_k[b, int(sp.index_absorb[0, b]) - 1]) if int(sp.n_band_absorb[b]) > 0 else 1
                for b in range(sp.n_band))
        lines["sw" if solar else "lw"] = {
            "value": world * N_COL * g / t_mx, "ms_per_step": t_mx * 1e3, "g_points": g,
            "fp64_value": world * N_COL * g / t_64, "fp64_ms_per_step": t_64 * 1e3,
            "max_flux_err_wm2": float(max(np.abs(o_mx[k] - o_64[k]).max() for k in ("flux_up", "flux_down"))),
            "max_heating_rate_err_kday": float(np.abs(o_mx["heating_rate"] - o_64["heating_rate"]).max())}
    if rank == 0:
        print(json.dumps({"metric": "column·g-points/s on the GA9 operational spectral files", "unit": UNIT,
                          "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                          "scaling": "weak", "dtype": "f32+f64", "data": "synthetic columns, GA9 spectral files",
                          "config": {"workload": f"GA9 LW and SW, lookup-table k, Wen-Yi, k_eqv_scl, continuum, "
                                                 f"{N_COL} columns x {N_LAYER} layers, clear sky",
                                     "l2": "256 MiB L2 flush between timed steps"},
                          "lw": lines["lw"], "sw": lines["sw"]}))


def main():
    args = parse()
    if args.steps is None:
        args.steps = 200
    if args.workload == "batched" and "--steps" in sys.argv and "--batched-steps" not in sys.argv:
        args.batched_steps = args.steps
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "batched":
        run_batched(args)
        return
    if args.workload == "serve":
        run_serve(args)
        return
    if args.workload == "ga9":
        run_ga9(args)
        return
    import numpy as np
    import torch
    rank, world = dist_setup(args.gpus)
    dev = torch.cuda.current_device()
    from socrates_gb300 import abi
    from socrates_gb300 import build as B
    from socrates_gb300 import radiance as R
    from socrates_gb300.device import DeviceCase
    from socrates_gb300.synth import config2
    if rank == 0:
        B.build()
    barrier(world)
    # each rank solves its own batch of columns (weak scaling, no exchange)
    sp, col = config2(N_COL, N_LAYER, SEED + rank)
    g = sp.n_gpoint
    ctl_mx = R.sw_control(l_aerosol_mode=True, precision=abi.PRECISION_MIXED)
    ctl_64 = R.sw_control(l_aerosol_mode=True, precision=abi.PRECISION_FP64)
    case = DeviceCase(ctl_mx, sp, col)
    case64 = DeviceCase(ctl_64, sp, col)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(c, steps, warm):
        for _ in range(warm):
            c.run(stream.cuda_stream)
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        l0 = R.launch_count()
        t0 = time.perf_counter()
        for e0, e1 in evs:
            flush.fill_(1.0)                 # evict L2 between steps (outside the events)
            e0.record(stream)
            c.run(stream.cuda_stream)
            e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        wall = time.perf_counter() - t0
        launches = R.launch_count() - l0
        ms = [e0.elapsed_time(e1) for e0, e1 in evs]
        return sum(ms) / steps, launches, wall

    with ClockSampler(dev) as clk:
        ms_mx, launches, wall = timed(case, args.steps, max(3, args.warmup))
    # the same step repeated for about a second, with clocks sampled over it:
    # the K timed steps above can be a few milliseconds only
    n_sus = max(args.steps, int(1000.0 / max(ms_mx, 1e-3)))
    with ClockSampler(dev) as clk_sus:
        ms_sus, _, wall_sus = timed(case, n_sus, 0)
    ms_64, _, _ = timed(case64, max(3, args.steps // 4), 3)
    ms_mx = max_over_ranks(ms_mx, world)
    ms_64 = max_over_ranks(ms_64, world)
    value = world * N_COL * g / (ms_mx * 1e-3)
    value_64 = world * N_COL * g / (ms_64 * 1e-3)

    # accuracy of the mixed path against the FP64 path on this batch
    err_flux = max(float(np.abs(case.output(k) - case64.output(k)).max())
                   for k in ("flux_up", "flux_down", "flux_direct"))
    err_hr = float(np.abs(case.output("heating_rate") - case64.output("heating_rate")).max())

    # end to end through the public host-pointer API (pinned host buffers)
    def pinned_copy(a):
        t = torch.empty(a.size, dtype=torch.float64).pin_memory()
        v = t.numpy().reshape(a.shape, order="F")
        v[...] = a
        return v, t
    keep = []
    for name in ("p", "t", "t_level", "mass", "gas_mix_ratio", "zen_0", "solar_irrad", "rho_alb"):
        v, t = pinned_copy(np.asfortranarray(getattr(col, name)))
        keep.append(t)
        setattr(col, name, v)
    for k in ("mode_mix_ratio", "mode_absorption", "mode_scattering", "mode_asymmetry"):
        v, t = pinned_copy(np.asfortranarray(col.aer[k]))
        keep.append(t)
        col.aer[k] = v
    import ctypes as C
    marsh = R.Marshal(ctl_mx, sp, col)
    for name in ("flux_up", "flux_down", "flux_direct", "flux_div", "heating_rate"):
        arr = getattr(marsh, name)
        v, t = pinned_copy(arr)
        keep.append(t)
        setattr(marsh, name, v)
        setattr(marsh.radout, name, v.ctypes.data_as(C.POINTER(C.c_double)))
    h = R.register_spectrum(sp)
    lib = R.load_library()
    msg = C.create_string_buffer(256)
    for _ in range(3):
        lib.socgpu_radiance_calc(*marsh.args(h), msg, 256)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = lib.socgpu_radiance_calc(*marsh.args(h), msg, 256)
        if st != 0:
            raise SystemExit(f"radiance_calc failed: {msg.value.decode()}")
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
    # t_ground and t_level are not read on the solar path
    h2d = case.input_bytes - case.tensor_bytes("t_ground") - case.tensor_bytes("t_level")
    d2h = case.output_bytes
    e2e = {"value": world * N_COL * g / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
           "path": "socgpu_radiance_calc with pinned host arrays (H2D inputs, kernel, D2H outputs)"}

    peak, peak_kind = measured_peak_hbm()
    alg_bytes = h2d + d2h
    achieved = alg_bytes / (ms_mx * 1e-3) / 1e9
    prof = profile_figures()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": prof.get("dram_bytes_per_launch"),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "algorithmic_bytes_per_launch": int(alg_bytes),
                "note": "compulsory FP64 I/O of the batch (inputs the solar kernel reads + outputs) over the "
                        "mixed kernel's CUDA-event time; the kernel is issue-bound, see issue_roofline"}
    if "warp_instructions_per_launch" in prof:
        sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
        clk_ghz = (clk.summary()["sm_mhz"] or 2070.0) / 1e3
        issue_peak = sm_count * 4 * clk_ghz          # warp instructions per ns: 4 schedulers per SM
        issue_achieved = prof["warp_instructions_per_launch"] / (ms_mx * 1e6)
        roofline["issue_roofline"] = {
            "achieved": issue_achieved, "peak": issue_peak, "unit": "G warp-instructions/s",
            "frac": issue_achieved / issue_peak,
            "note": "warp instructions per launch from the committed ncu summary over the live CUDA-event "
                    "time; peak = SMs x 4 issue slots x median SM clock sampled during the timed region"}
    if rank == 0:
        cpu = cpu_baseline(args.cpu_sample, args.cpu_seconds)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": max(3, args.warmup), "ms_per_step": ms_mx, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic (seeded Philox inputs with the workload's shapes and distributions)",
                "config": CONFIG, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
                "fp64_device": {"value": value_64, "ms_per_step": ms_64, "speedup_mixed_over_fp64": ms_64 / ms_mx},
                "accuracy_vs_fp64": {"max_flux_err_wm2": err_flux, "max_heating_rate_err_kday": err_hr},
                "gpu_launches": int(launches), "clocks": clk.summary(), "wall_s_timed_region": wall,
                "sustained": {"steps": n_sus, "ms_per_step": ms_sus, "wall_s": wall_sus, "clocks": clk_sus.summary(),
                              "note": "the timed step repeated for about 1 s (L2 flushed between steps)"}}
        if world == 1 and not args.no_extras:
            # the multi-batch graph (4096 uneven batches) and the serving
            # loop, measured in the same run and reported beside the headline
            del case, case64
            torch.cuda.empty_cache()
            line["batched"] = batched_figures(args)
            sv = serve_figures(args)
            line["serve"] = sv["results"]
            line["serve_fp64_per_request"] = sv["fp64_per_request"]
            line["serve_cpu_baseline"] = sv["cpu_baseline"]
            line["serve_config"] = sv["config"]
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
