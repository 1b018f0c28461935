"""Seeded synthetic workloads of many uneven radiance_calc requests.

A request is one column batch.  Its kind is LW or SW, clear or all-sky
(McICA), and it has a layer count from {38, 60, 85, 137}.  Its column count
is log-normal: median 256, log-space standard deviation 1, clipped to
1..8192.  The arrays of a request are a window of a pool: one synthetic
atmosphere per (kind, layer count), generated once.  So thousands of
requests cost a handful of generator calls.  Each request still gets its own
device copy of its inputs and its own outputs.

Kinds:
  lw_clear   -- infra-red, no scattering (Elsasser), as the LW clear workload
  sw_clear   -- solar PIFM80 delta-Eddington with Rayleigh
  lw_cloudy  -- infra-red with McICA clouds (16 subcolumns, exponential-random)
  sw_cloudy  -- solar with McICA clouds
"""
from __future__ import annotations

from dataclasses import dataclass, replace

import numpy as np

from . import abi, synth
from . import radiance as R

KINDS = ("lw_clear", "sw_clear", "lw_cloudy", "sw_cloudy")
LAYERS = (38, 60, 85, 137)
N_SUBCOL = 16


@dataclass
class RequestSpec:
    kind: str
    n_layer: int
    n_profile: int
    position: float    # where the request's window sits in its pool, 0..1
    offset: int = 0    # first column of the window (set by Pools)


def request_specs(n_request: int, seed: int, median: float = 256.0, sigma: float = 1.0,
                  clip: tuple[int, int] = (1, 8192)) -> list[RequestSpec]:
    rng = np.random.default_rng(seed)
    kinds = rng.integers(0, len(KINDS), n_request)
    layers = rng.integers(0, len(LAYERS), n_request)
    cols = np.clip(np.rint(rng.lognormal(np.log(median), sigma, n_request)), clip[0], clip[1]).astype(int)
    u = rng.random(n_request)
    return [RequestSpec(KINDS[k], LAYERS[l], int(n), float(f)) for k, l, n, f in zip(kinds, layers, cols, u)]


class Pools:
    """One synthetic atmosphere (and McICA state) per (kind, layer count),
    wide enough for the widest request of that key."""

    def __init__(self, specs: list[RequestSpec], seed: int):
        self.lw = synth.lw_spectrum(seed, 9, clouds=True)
        self.sw = synth.sw_spectrum(seed, 8, clouds=True)
        species = np.array(sorted(set(self.lw.type_absorb) | set(self.sw.type_absorb)), np.int32)
        width: dict[tuple[str, int], int] = {}
        for s in specs:
            key = (s.kind, s.n_layer)
            width[key] = max(width.get(key, 0), s.n_profile)
        self.pool = {}
        for i, (key, n) in enumerate(sorted(width.items())):
            kind, L = key
            ps = seed * 1000 + i
            col = synth.atmosphere(n, L, species, ps)
            sp = self.sw if kind.startswith("sw") else self.lw
            if kind.startswith("sw"):
                synth.add_sw_surface(col, sp.n_band, ps)
            else:
                synth.add_lw_surface(col, sp.n_band)
            mc = None
            if kind.endswith("cloudy"):
                synth.add_clouds(col, ps, N_SUBCOL)
                c_sub, nsc = R.cloud_gen(col, N_SUBCOL, abi.IP_EXPONENTIAL_RAND, abi.RNG_PHILOX)
                isolir = abi.IP_SOLAR if kind.startswith("sw") else abi.IP_INFRA_RED
                mc = R.set_cld_mcica(sp, col, isolir, abi.IP_MCICA_SINGLE_SAMPLING, c_sub=c_sub, n_subcol_cld=nsc)
            self.pool[key] = (sp, col, mc)
        for s in specs:
            n_pool = self.pool[(s.kind, s.n_layer)][1].n_profile
            s.offset = min(int(s.position * (n_pool - s.n_profile + 1)), n_pool - s.n_profile)

    @staticmethod
    def control(kind: str, precision: int) -> R.Control:
        if kind == "lw_clear":
            return R.lw_noscat_control(precision=precision)
        if kind == "sw_clear":
            return R.sw_control(precision=precision)
        if kind == "lw_cloudy":
            return R.lw_control(i_cloud=abi.IP_CLOUD_MCICA, precision=precision)
        return R.sw_control(i_cloud=abi.IP_CLOUD_MCICA, precision=precision)

    def request(self, s: RequestSpec, precision: int, alloc=None):
        """(control, spectrum, column, mcica) of one request; `alloc(shape,
        dtype)` places the request's arrays (e.g. PinnedArena.take)."""
        sp, col, mc = self.pool[(s.kind, s.n_layer)]
        c = synth.window(col, s.offset, s.n_profile, alloc)
        m = None
        if mc is not None:
            sl = slice(s.offset, s.offset + s.n_profile)

            def cut(v):
                if alloc is None:
                    return np.asfortranarray(v[sl]) if v.ndim > 1 else np.ascontiguousarray(v[sl])
                out = alloc(v[sl].shape, v.dtype)
                out[...] = v[sl]
                return out
            m = replace(mc, c_sub=cut(mc.c_sub), n_subcol_cld=cut(mc.n_subcol_cld), frac_cloudy=cut(mc.frac_cloudy))
        return self.control(s.kind, precision), sp, c, m


class PinnedArena:
    """Page-locked host memory handed out as Fortran-ordered numpy arrays
    (bump allocation; freed as a whole)."""

    def __init__(self, nbytes: int):
        import torch
        self._buf = torch.empty(int(nbytes), dtype=torch.uint8, pin_memory=True)
        self._mem = self._buf.numpy()
        self._off = 0

    def take(self, shape, dtype) -> np.ndarray:
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        off = (self._off + 255) & ~255
        if off + n > self._mem.size:
            raise MemoryError("pinned arena exhausted")
        self._off = off + n
        return np.ndarray(shape, dtype=dtype, buffer=self._mem, offset=off, order="F")

    def reset(self) -> None:
        self._off = 0


def pin_outputs(m: R.Marshal, alloc) -> R.Marshal:
    """Point a Marshal's outputs at arrays from `alloc` (page-locked)."""
    import ctypes as C
    dp = C.POINTER(C.c_double)
    for name in ("flux_up", "flux_down", "flux_direct", "flux_div", "heating_rate"):
        a = getattr(m, name)
        if a is None:
            continue
        b = alloc(a.shape, a.dtype)
        b[...] = 0.0
        setattr(m, name, b)
        setattr(m.radout, name, b.ctypes.data_as(dp))
    return m


def n_gpoint(kind: str) -> int:
    return 81 if kind.startswith("lw") else 48
