"""Host-side mirror of the reference's radiance_calc / set_cld_mcica / cloud_gen
interfaces, calling libsocgpu through its C-ABI.

``radiance_calc(control, spectrum, col, ...)`` takes the same option ids and
arrays as src/radiance_core/radiance_calc.F90:16 (through the Column
container of synth.py, which holds atm/bound/aer/cld fields in the
reference's Fortran layouts) and returns the StrOut fluxes.  Errors come
back as RadianceError carrying the reference's status code; there is no
host fallback: a missing or unloadable library raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from dataclasses import dataclass, field, replace
from pathlib import Path

import numpy as np

from . import abi
from .spectrum import Spectrum

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libsocgpu.so"


class RadianceError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"status {status}: {message}")
        self.status = status
        self.message = message


_lib = None
_lib_lock = threading.Lock()


def load_library(path: Path | None = None) -> C.CDLL:
    """Load libsocgpu.so (raises if it is missing: there is no fallback)."""
    global _lib
    with _lib_lock:
        if _lib is None:
            p = Path(path) if path else LIB_PATH
            if not p.exists():
                raise RuntimeError(f"{p} is missing: build it with socrates_gb300.build.build()")
            _lib = abi.declare(C.CDLL(str(p)))
            if _lib.socgpu_abi_version() != abi.ABI_VERSION:
                raise RuntimeError("libsocgpu ABI version mismatch")
    return _lib


# ---------------------------------------------------------------------------
@dataclass
class Control:
    """StrCtrl subset with the defaults socrates_set_control.F90:246-375
    gives the two-stream path (SW: PIFM80 + full scattering; LW: Elsasser,
    quadratic source)."""
    isolir: int = abi.IP_INFRA_RED
    i_2stream: int = abi.IP_ELSASSER
    i_scatter_method: int = abi.IP_SCATTER_FULL
    i_solver: int = abi.IP_SOLVER_HOMOGEN_DIRECT
    i_cloud: int = abi.IP_CLOUD_CLEAR
    i_gas_overlap: int = abi.IP_OVERLAP_RANDOM
    i_direct_tau: int = abi.IP_DIRECT_DELTA_SCALING
    l_rescale: bool = True
    n_order_forward: int = 2
    l_ir_source_quad: bool = True
    l_rayleigh: bool = False
    l_gas: bool = True
    l_aerosol_mode: bool = False
    l_flux_div: bool = True
    first_band: int = 1
    last_band: int = 0           # 0: all bands
    weight_band: np.ndarray | None = None
    precision: int = abi.PRECISION_FP64
    l_continuum: bool = False
    l_mixing_ratio: bool = False
    l_grey_single: bool = False
    l_aerosol: bool = False
    l_henyey_greenstein_pf: bool = False
    # how the cloud types group into regions (the three-region scheme needs
    # conv_strat, csiw or a split representation)
    i_cloud_representation: int = abi.IP_CLOUD_ICE_WATER

    def as_struct(self, n_band: int, keep: list) -> abi.Control:
        c = abi.Control()
        c.isolir, c.i_angular_integration, c.i_2stream = self.isolir, abi.IP_TWO_STREAM, self.i_2stream
        c.i_scatter_method, c.i_solver, c.i_cloud = self.i_scatter_method, self.i_solver, self.i_cloud
        c.i_cloud_representation = self.i_cloud_representation
        c.i_gas_overlap, c.i_direct_tau = self.i_gas_overlap, self.i_direct_tau
        c.l_rescale, c.n_order_forward = int(self.l_rescale), self.n_order_forward
        c.l_ir_source_quad, c.l_rayleigh, c.l_gas = int(self.l_ir_source_quad), int(self.l_rayleigh), int(self.l_gas)
        c.l_aerosol_mode, c.l_flux_div = int(self.l_aerosol_mode), int(self.l_flux_div)
        c.first_band = self.first_band
        c.last_band = self.last_band if self.last_band > 0 else n_band
        c.weight_band = _dp(self.weight_band, keep)
        c.precision = self.precision
        c.l_continuum, c.l_mixing_ratio = int(self.l_continuum), int(self.l_mixing_ratio)
        c.l_grey_single = int(self.l_grey_single)
        c.l_aerosol, c.l_henyey_greenstein_pf = int(self.l_aerosol), int(self.l_henyey_greenstein_pf)
        return c


def lw_control(**kw) -> Control:
    return replace(Control(isolir=abi.IP_INFRA_RED, i_2stream=abi.IP_ELSASSER), **kw)


def lw_noscat_control(**kw) -> Control:
    """Plain longwave clear sky: no scattering, Elsasser diffusivity 1.66."""
    return replace(Control(isolir=abi.IP_INFRA_RED, i_2stream=abi.IP_ELSASSER,
                           i_scatter_method=abi.IP_NO_SCATTER_ABS, i_solver=abi.IP_SOLVER_NO_SCAT), **kw)


def sw_control(**kw) -> Control:
    return replace(Control(isolir=abi.IP_SOLAR, i_2stream=abi.IP_PIFM80, l_rayleigh=True,
                           l_ir_source_quad=False), **kw)


def _dp(a, keep):
    if a is None:
        return None
    a = np.asfortranarray(a, dtype=np.float64)
    keep.append(a)
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a, keep):
    if a is None:
        return None
    a = np.asfortranarray(a, dtype=np.int32)
    keep.append(a)
    return a.ctypes.data_as(C.POINTER(C.c_int))


@dataclass
class McicaState:
    """What set_cld_mcica (socrates_set_cld_mcica.F90:82-228) leaves in cld
    for the two-stream solve."""
    n_subcol_gen: int
    n_subcol_req: int
    c_sub: np.ndarray            # (n_profile, L - id_ct + 1, n_subcol_gen), compacted (cloud_gen)
    n_subcol_cld: np.ndarray     # (n_profile)
    frac_cloudy: np.ndarray      # (n_profile)
    subcol_k: np.ndarray         # (n_band, nd_k_term)
    first_subcol_k: np.ndarray   # (n_band, nd_k_term + 1)
    subcol_reorder: np.ndarray   # (n_subcol_req)


@dataclass
class McicaData:
    """The McICA data file of a pair of spectral files (StrMcica,
    def_mcica.F90): subcolumn counts, the sampling tables and the table of
    the water-content distribution for cloud_gen."""
    n_subcol_gen: int = 0
    n_subcol_req_single: int = 0
    n_subcol_req_optimal: int = 0
    ipph: int = 0
    lw_subcol_reorder_single: np.ndarray | None = None
    lw_subcol_reorder_optimal: np.ndarray | None = None
    sw_subcol_k: dict | None = None      # {(band, k): subcolumns}, 1-based; others take 1
    lw_subcol_k: dict | None = None
    xcw: np.ndarray | None = None        # (n1, n2)


def read_mcica_data(path) -> McicaData:
    """read_mcica_data (def_mcica.F90): the keyword records of the *DATA
    block, each followed by its values."""
    lines = open(path).read().splitlines()
    i = next(q for q, ln in enumerate(lines) if ln.startswith("*DATA")) + 1
    d = McicaData()
    n1 = n2 = 0

    def numbers(start, count, conv=int):
        out, q = [], start
        while len(out) < count:
            out += [conv(x) for x in lines[q].split()]
            q += 1
        return out[:count], q

    while i < len(lines) and not lines[i].startswith("*END"):
        key = lines[i].strip()
        i += 1
        if key in ("tot_subcol_gen", "n_subcol_gen"):
            (d.n_subcol_gen,), i = numbers(i, 1)
        elif key in ("subcol_need_single", "n_subcol_req_single"):
            (d.n_subcol_req_single,), i = numbers(i, 1)
        elif key in ("subcol_need_optimal", "n_subcol_req_optimal"):
            (d.n_subcol_req_optimal,), i = numbers(i, 1)
        elif key == "ipph":
            (d.ipph,), i = numbers(i, 1)
        elif key == "lw_subcol_reorder_single":
            v, i = numbers(i, d.n_subcol_req_single)
            d.lw_subcol_reorder_single = np.array(v, np.int32)
        elif key == "lw_subcol_reorder_optimal":
            v, i = numbers(i, d.n_subcol_req_optimal)
            d.lw_subcol_reorder_optimal = np.array(v, np.int32)
        elif key in ("sw_subcol_k", "lw_subcol_k"):
            table = {}
            while True:
                b, k, n = (int(x) for x in lines[i].split()[:3])
                i += 1
                if b == -99:
                    break
                table[(b, k)] = n
            setattr(d, key, table)
        elif key == "n1":
            (n1,), i = numbers(i, 1)
        elif key == "n2":
            (n2,), i = numbers(i, 1)
        elif key == "xcw":
            v, i = numbers(i, n1 * n2, float)
            d.xcw = np.asfortranarray(np.array(v).reshape((n1, n2), order="F"))
    return d


def write_mcica_data(path, d: McicaData) -> None:
    """The McICA data file in the record layout read_mcica_data reads."""
    L = ["*DATA", "", "tot_subcol_gen", f"{d.n_subcol_gen:5d}", "subcol_need_single", f"{d.n_subcol_req_single:5d}",
         "subcol_need_optimal", f"{d.n_subcol_req_optimal:5d}", "ipph", f"{d.ipph:5d}", ""]
    rows = lambda v, fmt, n: ["".join(fmt.format(x) for x in v[q:q + n]) for q in range(0, len(v), n)]
    for key in ("lw_subcol_reorder_single", "lw_subcol_reorder_optimal"):
        v = getattr(d, key)
        if v is not None:
            L += [key] + rows(list(v), "{:5d}", 10) + [""]
    for key in ("sw_subcol_k", "lw_subcol_k"):
        L.append(key)
        L += [f"{b:4d}{k:4d}{n:4d}" for (b, k), n in sorted((getattr(d, key) or {}).items())]
        L += [f"{-99:4d}{0:4d}{0:4d}", ""]
    n1, n2 = d.xcw.shape
    L += ["n1", f"{n1:6d}", "n2", f"{n2:6d}", "xcw"]
    L += rows(list(d.xcw.ravel(order="F")), " {:15.8E}", 5)
    L.append("*END")
    with open(path, "w") as fh:
        fh.write("\n".join(L) + "\n")


def mcica_sampling(spectrum: Spectrum, isolir: int, n_subcol_gen: int, sampling: int, first_band: int = 1,
                   last_band: int = 0, data: McicaData | None = None):
    """subcol_k, first_subcol_k, subcol_reorder and n_subcol_req of
    set_cld_mcica (socrates_set_cld_mcica.F90:106-160) with the counts of
    l_run_cdf.F90:1281-1290.  With the McICA data file, the tables are the
    reference's; without it single sampling takes one subcolumn per k-term
    with n_subcol_req = number of k-terms, and optimal sampling is refused."""
    nb, ndk = spectrum.n_band, spectrum.nd_k_term
    last_band = last_band or nb
    if data is not None and sampling != abi.IP_MCICA_FULL_SAMPLING:
        single = sampling == abi.IP_MCICA_SINGLE_SAMPLING
        req = data.n_subcol_req_single if single else data.n_subcol_req_optimal
        subcol_k = np.ones((nb, ndk), np.int32)
        if not single:
            table = data.sw_subcol_k if isolir == abi.IP_SOLAR else data.lw_subcol_k
            for (b, k), n in (table or {}).items():
                if 1 <= b <= nb and 1 <= k <= ndk:
                    subcol_k[b - 1, k - 1] = n
        if isolir == abi.IP_SOLAR:
            reorder = np.array([l % n_subcol_gen for l in range(1, req + 1)], np.int32)
        else:
            src = data.lw_subcol_reorder_single if single else data.lw_subcol_reorder_optimal
            reorder = np.asarray(src[:req], np.int32) % n_subcol_gen
        reorder[reorder == 0] = n_subcol_gen
        return np.asfortranarray(subcol_k), _first_subcol(spectrum, subcol_k, first_band, last_band), reorder, req
    if sampling == abi.IP_MCICA_FULL_SAMPLING:
        subcol_k = np.full((nb, ndk), n_subcol_gen, np.int32)
        req = n_subcol_gen
    elif sampling == abi.IP_MCICA_SINGLE_SAMPLING:
        subcol_k = np.ones((nb, ndk), np.int32)
        req = 0
        for b in range(first_band - 1, last_band):
            g = int(spectrum.index_absorb[0, b]) - 1
            req += int(spectrum.i_band_k[b, g])
        req = max(req, 1)
    else:
        raise RadianceError(abi.I_ERR_FATAL, "optimal sampling needs the reference's mcica_data tables")
    first = _first_subcol(spectrum, subcol_k, first_band, last_band)
    if isolir == abi.IP_SOLAR or sampling != abi.IP_MCICA_FULL_SAMPLING:
        reorder = np.array([l % n_subcol_gen for l in range(1, req + 1)], np.int32)
    else:
        reorder = np.arange(1, req + 1, dtype=np.int32)
    reorder[reorder == 0] = n_subcol_gen
    return np.asfortranarray(subcol_k), np.asfortranarray(first), reorder, req


def _first_subcol(spectrum: Spectrum, subcol_k, first_band: int, last_band: int):
    """first_subcol_k (socrates_set_cld_mcica.F90:129-139)."""
    nb, ndk = spectrum.n_band, spectrum.nd_k_term
    first = np.zeros((nb, ndk + 1), np.int32)
    first[first_band - 1, 0] = 1
    for b in range(first_band - 1, last_band):
        g = int(spectrum.index_absorb[0, b]) - 1
        n_k = int(spectrum.i_band_k[b, g])
        for k in range(n_k):
            first[b, k + 1] = first[b, k] + subcol_k[b, k]
        if b < last_band - 1:
            first[b + 1, 0] = first[b, n_k]
    return np.asfortranarray(first)


# ---------------------------------------------------------------------------
class Marshal:
    """Builds the C structures of one radiance_calc call from numpy arrays."""

    def __init__(self, control: Control, spectrum: Spectrum, col, mcica: McicaState | None = None,
                 id_cloud_top: int = 1, alloc=None):
        self.keep: list = []
        k = self.keep
        n, L = col.n_profile, col.n_layer
        self.n, self.L = n, L
        self.control = control.as_struct(spectrum.n_band, k)
        d = abi.Dimen()
        d.nd_profile, d.nd_layer, d.id_cloud_top = n, L, id_cloud_top
        d.nd_aerosol_mode = col.aer["n_mode"] if (col.aer and control.l_aerosol_mode) else 1
        d.nd_cloud_component, d.nd_cloud_type = 2, 2
        d.nd_subcol_gen = mcica.n_subcol_gen if mcica else 1
        d.nd_subcol_req = mcica.n_subcol_req if mcica else 1
        self.dimen = d
        a = abi.Atm()
        a.n_profile, a.n_layer = n, L
        a.p, a.t = _dp(col.p, k), _dp(col.t, k)
        a.p_level, a.t_level = _dp(col.p_level, k), _dp(col.t_level, k)
        a.mass, a.gas_mix_ratio = _dp(col.mass, k), _dp(col.gas_mix_ratio, k)
        a.density = _dp(getattr(col, "density", None), k)
        self.atm = a
        b = abi.Bound()
        b.zen_0, b.solar_irrad = _dp(col.zen_0, k), _dp(col.solar_irrad, k)
        b.rho_alb, b.t_ground = _dp(col.rho_alb, k), _dp(col.t_ground, k)
        b.flux_ground = _dp(getattr(col, "flux_ground", None), k)
        self.bound = b
        self.aer = abi.Aer()
        if control.l_aerosol_mode and col.aer:
            ae = col.aer
            self.aer.n_mode = ae["n_mode"]
            self.aer.mode_mix_ratio = _dp(ae["mode_mix_ratio"], k)
            self.aer.mode_absorption = _dp(ae["mode_absorption"], k)
            self.aer.mode_scattering = _dp(ae["mode_scattering"], k)
            self.aer.mode_asymmetry = _dp(ae["mode_asymmetry"], k)
        # classic aerosol: col.aer["mix_ratio"] (n, L, n_entries) of the
        # spectral file's species "mr_type_index" (1-based), with optional
        # "mr_source" and, for moist species, "mean_rel_humidity" (n, L)
        d.nd_aerosol_mr = 1
        if control.l_aerosol and col.aer and "mix_ratio" in col.aer:
            ae = col.aer
            mr = ae["mix_ratio"]
            self.aer.n_aerosol_mr = int(mr.shape[2])
            d.nd_aerosol_mr = max(1, int(mr.shape[2]))
            self.aer.mix_ratio = _dp(mr, k)
            self.aer.mr_type_index = _ip(ae["mr_type_index"], k)
            self.aer.mr_source = _ip(ae.get("mr_source"), k)
            self.aer.mean_rel_humidity = _dp(ae.get("mean_rel_humidity"), k)
            # prescribed properties of unparametrized species: "pressure_prsc"
            # (n, levels, species), "absorption_prsc"/"scattering_prsc" (n,
            # levels, species, bands), "phase_fnc_prsc" (n, levels, moments,
            # species, bands), "n_opt_level_prsc" and "n_phase_term_prsc"
            # (species)
            if "pressure_prsc" in ae:
                ph = ae["phase_fnc_prsc"]
                d.nd_profile_aerosol_prsc, d.nd_opt_level_aerosol_prsc = ph.shape[0], ph.shape[1]
                d.nd_phf_term_aerosol_prsc = ph.shape[2]
                self.aer.n_opt_level_prsc = _ip(ae["n_opt_level_prsc"], k)
                self.aer.n_phase_term_prsc = _ip(ae["n_phase_term_prsc"], k)
                self.aer.pressure_prsc = _dp(ae["pressure_prsc"], k)
                self.aer.absorption_prsc = _dp(ae["absorption_prsc"], k)
                self.aer.scattering_prsc = _dp(ae["scattering_prsc"], k)
                self.aer.phase_fnc_prsc = _dp(ph, k)
        self.cld = abi.Cld()
        region = control.i_cloud in (abi.IP_CLOUD_MIX_MAX, abi.IP_CLOUD_MIX_RANDOM, abi.IP_CLOUD_TRIPLE,
                                     abi.IP_CLOUD_PART_CORR, abi.IP_CLOUD_PART_CORR_CNV)
        if mcica is not None or (region and col.cld):
            cd = col.cld
            ict = id_cloud_top - 1
            cl = self.cld
            # components: water and ice as two cloud types with the Pade
            # schemes of type 1 unless the cloud fields say otherwise
            cl.n_condensed = int(cd.get("n_condensed", 2))
            cl.type_condensed = _ip(cd.get("type_condensed", [abi.IP_PHASE_WATER, abi.IP_PHASE_ICE]), k)
            cl.i_cloud_type = _ip(cd.get("i_cloud_type", [abi.IP_CLOUD_TYPE_WATER, abi.IP_CLOUD_TYPE_ICE]), k)
            cl.i_condensed_param = _ip(cd.get("i_condensed_param", [abi.IP_DROP_PADE_2, abi.IP_ICE_PADE_2_PHF]), k)
            cl.i_condensed_type = _ip(cd.get("i_condensed_type", [1, 1]), k)
            cl.condensed_mix_ratio = _dp(cd["condensed_mix_ratio"][:, ict:, :], k)
            cl.condensed_dim_char = _dp(cd["condensed_dim_char"][:, ict:, :], k)
            cl.n_cloud_type = int(cd.get("n_cloud_type", 2))
            # the extents of the arrays as given (the host path copies them whole)
            self.dimen.nd_cloud_component, self.dimen.nd_cloud_type = cl.n_condensed, cl.n_cloud_type
            cl.w_cloud = _dp(cd["w_cloud"][:, ict:], k)
            cl.frac_cloud = _dp(cd["frac_cloud"][:, ict:, :], k)
            cl.dp_corr_strat = float(cd.get("dp_corr_strat", 0.0))
            cl.dp_corr_conv = float(cd.get("dp_corr_conv", 0.0))
            if mcica is not None:
                cl.n_subcol_gen, cl.n_subcol_req = mcica.n_subcol_gen, mcica.n_subcol_req
                cl.c_sub = _dp(mcica.c_sub, k)
                cl.frac_cloudy = _dp(mcica.frac_cloudy, k)
                cl.n_subcol_cld = _ip(mcica.n_subcol_cld, k)
                cl.subcol_k = _ip(mcica.subcol_k, k)
                cl.first_subcol_k = _ip(mcica.first_subcol_k, k)
                cl.subcol_reorder = _ip(mcica.subcol_reorder, k)
        # outputs from `alloc(*shape)` (F-ordered zeros), e.g. page-locked
        f = alloc or (lambda *s: np.zeros(s, order="F"))
        self.flux_up, self.flux_down = f(n, L + 1), f(n, L + 1)
        self.flux_direct = f(n, L + 1) if control.isolir == abi.IP_SOLAR else None
        self.flux_div = f(n, L) if control.l_flux_div else None
        self.heating_rate = f(n, L)
        r = abi.Radout()
        r.flux_up = self.flux_up.ctypes.data_as(C.POINTER(C.c_double))
        r.flux_down = self.flux_down.ctypes.data_as(C.POINTER(C.c_double))
        r.flux_direct = None if self.flux_direct is None else self.flux_direct.ctypes.data_as(C.POINTER(C.c_double))
        r.flux_div = None if self.flux_div is None else self.flux_div.ctypes.data_as(C.POINTER(C.c_double))
        r.heating_rate = self.heating_rate.ctypes.data_as(C.POINTER(C.c_double))
        self.radout = r

    def args(self, handle_or_desc):
        return (C.byref(self.control), C.byref(self.dimen), handle_or_desc, C.byref(self.atm), C.byref(self.cld),
                C.byref(self.aer), C.byref(self.bound), C.byref(self.radout))

    def result(self) -> dict:
        out = dict(flux_up=self.flux_up, flux_down=self.flux_down, heating_rate=self.heating_rate)
        if self.flux_direct is not None:
            out["flux_direct"] = self.flux_direct
        if self.flux_div is not None:
            out["flux_div"] = self.flux_div
        return out


# ---------------------------------------------------------------------------
_handles: dict[str, int] = {}


def register_spectrum(spectrum: Spectrum) -> int:
    """Device-resident spectral tables keyed by name
    (socrates_set_spectrum.F90:20-23,90-121)."""
    lib = load_library()
    if spectrum.name in _handles:
        return _handles[spectrum.name]
    desc = spectrum.to_desc()
    h = C.c_int(0)
    msg = C.create_string_buffer(512)
    st = lib.socgpu_spectrum_register(spectrum.name.encode(), C.byref(desc), C.byref(h), msg, 512)
    if st != abi.I_NORMAL:
        raise RadianceError(st, msg.value.decode())
    _handles[spectrum.name] = h.value
    return h.value


def radiance_calc(control: Control, spectrum: Spectrum, col, mcica: McicaState | None = None,
                  id_cloud_top: int = 1) -> dict:
    """radiance_calc on the GPU through socgpu_radiance_calc (host arrays)."""
    lib = load_library()
    h = register_spectrum(spectrum)
    m = Marshal(control, spectrum, col, mcica, id_cloud_top)
    msg = C.create_string_buffer(512)
    st = lib.socgpu_radiance_calc(*m.args(h), msg, 512)
    if st != abi.I_NORMAL:
        raise RadianceError(st, msg.value.decode())
    return m.result()


def cloud_gen(col, n_subcol: int, ioverlap: int = abi.IP_EXPONENTIAL_RAND, rng: int = abi.RNG_LCG,
              id_cloud_top: int = 1, ipph: int = 0, xcw: np.ndarray | None = None, sigma_qcw=None,
              impl=None):
    """cloud_gen (socrates_cloud_gen.F90:8-470) on the GPU; returns
    (c_sub, n_subcol_cld).  `impl` selects another library exporting the
    same signature (the tests pass the oracle)."""
    cd = col.cld
    n, L = col.n_profile, col.n_layer
    ict = id_cloud_top - 1
    keep: list = []
    ndc = L - ict
    c_sub = np.zeros((n, ndc, n_subcol), order="F")
    nsc = np.zeros(n, np.int32)
    zero = np.zeros((n, ndc), order="F")
    sig = zero if sigma_qcw is None else sigma_qcw
    xc = np.zeros((2, 2), order="F") if xcw is None else xcw
    seeds = np.ascontiguousarray(cd["rand_seed"], dtype=np.int32)
    args = [L, id_cloud_top, L, n, 1, n, n_subcol, xc.shape[0], xc.shape[1], ipph, ioverlap,
            seeds.ctypes.data, _dp(cd["dp_corr_cloud"][:, ict:], keep), _dp(cd["dp_corr_cond"][:, ict:], keep),
            _dp(sig, keep), _dp(cd["w_cloud"][:, ict:], keep), _dp(zero, keep), _dp(zero, keep),
            _dp(col.p, keep), _dp(xc, keep), nsc.ctypes.data, c_sub.ctypes.data, rng]
    args = [a if not isinstance(a, C._Pointer) else C.cast(a, C.c_void_p) for a in args]
    if impl is None:
        lib = load_library()
        msg = C.create_string_buffer(512)
        st = lib.socgpu_cloud_gen(*args, msg, 512)
        if st != abi.I_NORMAL:
            raise RadianceError(st, msg.value.decode())
    else:
        st = impl(*args)
        if st != abi.I_NORMAL:
            raise RadianceError(st, "cloud_gen failed")
    return c_sub, nsc


def set_cld_mcica(spectrum: Spectrum, col, isolir: int, sampling: int = abi.IP_MCICA_SINGLE_SAMPLING,
                  ioverlap: int = abi.IP_EXPONENTIAL_RAND, rng: int = abi.RNG_LCG, id_cloud_top: int = 1,
                  c_sub=None, n_subcol_cld=None, data: McicaData | None = None, impl=None) -> McicaState:
    """set_cld_mcica (socrates_set_cld_mcica.F90:82-228): sampling tables,
    the generator and frac_cloudy; the fill of cloudy subcolumns is applied
    by the solver from n_subcol_cld.

    With the McICA data file (`data`) the call is the reference's: its
    subcolumn counts and tables, the generator's ipph and xcw, the relative
    standard deviation of each component (col.cld["rel_var_dens"]) combined
    with the grid-box condensate as weights, and the condensate decorrelation
    at half the cloud's (lines 165-193)."""
    cd = col.cld
    gen = int(data.n_subcol_gen if data is not None else cd["n_subcol_gen"])
    subcol_k, first, reorder, req = mcica_sampling(spectrum, isolir, gen, sampling, data=data)
    if c_sub is None and data is not None:
        ict = id_cloud_top - 1
        nc = int(cd.get("n_condensed", 2))
        types = cd.get("i_cloud_type", [abi.IP_CLOUD_TYPE_WATER, abi.IP_CLOUD_TYPE_ICE])
        rvd = np.broadcast_to(np.asarray(cd.get("rel_var_dens", 0.0), dtype=np.float64), (nc,))
        eps = np.finfo(np.float64).eps
        num = np.zeros((col.n_profile, col.n_layer - ict))
        den = np.zeros_like(num)
        for i in range(nc):
            wgt = np.maximum(eps, cd["condensed_mix_ratio"][:, ict:, i] * cd["frac_cloud"][:, ict:, types[i] - 1])
            num = num + rvd[i] * wgt
            den = den + wgt
        cols = dict(cd)
        cols["dp_corr_cond"] = cd["dp_corr_cloud"] * 0.5
        col2 = type(col)(**{**col.__dict__, "cld": cols})
        c_sub, n_subcol_cld = cloud_gen(col2, gen, ioverlap, rng, id_cloud_top, ipph=data.ipph, xcw=data.xcw,
                                        sigma_qcw=np.asfortranarray(num / den), impl=impl)
    elif c_sub is None:
        c_sub, n_subcol_cld = cloud_gen(col, gen, ioverlap, rng, id_cloud_top, impl=impl)
    if sampling == abi.IP_MCICA_FULL_SAMPLING:
        frac_cloudy = np.ones(col.n_profile)
    else:
        frac_cloudy = n_subcol_cld.astype(np.float64) / float(gen)
    return McicaState(gen, req, c_sub, n_subcol_cld, frac_cloudy, subcol_k, first, reorder)


def launch_count() -> int:
    return int(load_library().socgpu_kernel_launch_count())
