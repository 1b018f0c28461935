"""Seeded synthetic spectral tables and atmospheres for the benchmark workloads.

No public dataset is named for this path, so the workloads are generated:
  * grid: level pressures log-spaced from 10 Pa (level 0, top) to 1e5 Pa
    (surface); layer pressure sqrt(p_{i-1} p_i); mass = dp/g; heights by the
    hypsometric equation;
  * temperature 288 K - 6.5 K/km down to 217 K, then isothermal, plus a
    per-column offset U(-10, 10) K;
  * H2O 1e-2 exp(-z/2 km) floored at 3e-6, times (1 + 0.3 U(-1, 1)) per
    column; CO2 6e-4; O3 a Gaussian in ln p, peak 1e-5 at 1000 Pa, width 1
    in ln p (the width is this generator's choice);
  * spectral tables: one absorber per band, k log-uniform 1e-4..1e2 m2/kg
    with power-law scaling (p/1e5 Pa)^0.75 (T/260 K)^1, weights summing to
    1 per band, band Planck flux a degree-5 polynomial in T/250 K fitted to
    the band-integrated Planck function, solar fractions from a 5778 K black
    body, Rayleigh coefficient 8.6e-7 m2/kg (lambda/1 um)^-4;
  * aerosol: one mode in the lowest 2 km, tau550 log-uniform 0.01..0.5,
    omega U(0.85, 0.99), g U(0.6, 0.75), Angstrom exponent 1.2;
  * clouds: 30 % of the layers below 100 hPa cloudy with fraction U(0, 1); liquid below 6 km
    (LWC log-normal, median 0.1 g/m3, sigma 1; re U(4, 16) um), ice above
    (IWC log-normal, median 0.02 g/m3, sigma 1; De U(20, 120) um); Pade
    optics with this generator's coefficient sets.
Random numbers are Philox4x32-10 streams keyed by (seed, stream id).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import abi
from .spectrum import Spectrum

GRAV = 9.80665          # rad_ccf.F90:50
R_DRY = 287.026         # rad_ccf.F90:54
SOLAR_CONSTANT = 1361.0
# Background mass mixing ratios of trace gases by identifier (N2O, CH4, O2,
# SO2, CFC11, CFC12, CFC113, HCFC22, HFC134a, OCS).
TRACE_MMR = {4: 4.8e-7, 6: 1.0e-6, 7: 0.231, 9: 1.0e-9, 14: 1.1e-9, 15: 2.3e-9, 16: 4.5e-10, 17: 7.5e-10,
             19: 2.8e-10, 25: 1.0e-9}

# ---------------------------------------------------------------------------
# Philox4x32-10, vectorised (Salmon et al., SC'11)
_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32(c0, c1, c2, c3, k0, k1):
    c0, c1, c2, c3 = (np.asarray(x, np.uint32) for x in (c0, c1, c2, c3))
    k0 = np.uint32(k0)
    k1 = np.uint32(k1)
    with np.errstate(over="ignore"):
        for _ in range(10):
            p0 = _M0 * c0.astype(np.uint64)
            p1 = _M1 * c2.astype(np.uint64)
            hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), (p0 & _MASK).astype(np.uint32)
            hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), (p1 & _MASK).astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
            k0 = np.uint32(k0 + _W0)
            k1 = np.uint32(k1 + _W1)
    return c0, c1, c2, c3


class Stream:
    """Uniform deviates in [0, 1) from Philox keyed by (seed, stream id)."""

    def __init__(self, seed: int, stream: int):
        self.seed = seed & 0xFFFFFFFF
        self.stream = stream & 0xFFFFFFFF
        self.counter = 0

    def uniform(self, shape) -> np.ndarray:
        n = int(np.prod(shape)) if shape != () else 1
        nblk = (n + 3) // 4
        idx = np.arange(self.counter, self.counter + nblk, dtype=np.uint64)
        self.counter += nblk
        w = philox4x32((idx & _MASK).astype(np.uint32), (idx >> np.uint64(32)).astype(np.uint32),
                       np.full(nblk, self.stream, np.uint32), np.zeros(nblk, np.uint32),
                       self.seed, 0x5EED0001)
        u = np.stack(w, axis=1).reshape(-1)[:n].astype(np.float64) * (1.0 / 4294967296.0)
        return u.reshape(shape)


# ---------------------------------------------------------------------------
def _planck_band(nu_lo, nu_hi, temps):
    """Band-integrated pi*B over wavenumbers nu_lo..nu_hi (cm-1) in W/m2."""
    h, c, kb = 6.62607015e-34, 2.99792458e8, 1.380649e-23
    nu = np.linspace(nu_lo, nu_hi, 2001) * 100.0  # m-1
    t = np.asarray(temps)[:, None]
    x = h * c * nu[None, :] / (kb * t)
    b = 2.0 * h * c ** 2 * nu[None, :] ** 3 / np.expm1(x)
    return np.pi * np.trapezoid(b, nu, axis=1)


def _kterms(st: Stream, nk: int):
    u = st.uniform((nk,))
    lk = -4.0 + 6.0 * (np.arange(nk) + 0.5 + 0.3 * (u - 0.5)) / nk
    k = 10.0 ** lk
    w = np.exp(-0.35 * np.arange(nk)) * (0.5 + st.uniform((nk,)))
    return k, w / w.sum()


def _base_spectrum(n_band, absorber_of_band, nk, st: Stream, wl_short, wl_long):
    species = sorted(set(absorber_of_band))
    n_abs = len(species)
    ia = np.zeros((n_abs, n_band), np.int32)
    nba = np.ones(n_band, np.int32)
    ibk = np.zeros((n_band, n_abs), np.int32)
    isk = np.zeros((n_band, n_abs), np.int32)
    isf = np.zeros((n_band, n_abs), np.int32)
    k = np.zeros((nk, n_band, n_abs))
    w = np.zeros((nk, n_band, n_abs))
    sc = np.zeros((2, nk, n_band, n_abs))
    pr = np.zeros((n_abs, n_band))
    tr = np.zeros((n_abs, n_band))
    for b, gas in enumerate(absorber_of_band):
        g = species.index(gas)
        ia[0, b] = g + 1
        ibk[b, g] = nk
        isk[b, g] = 1           # ip_scale_band
        isf[b, g] = 1           # ip_scale_power_law
        kk, ww = _kterms(st, nk)
        k[:, b, g] = kk
        w[:, b, g] = ww
        sc[0, :, b, g] = 0.75
        sc[1, :, b, g] = 1.0
        pr[g, b] = 1.0e5
        tr[g, b] = 260.0
    f = np.asfortranarray
    return dict(n_band=n_band, wavelength_short=np.array(wl_short), wavelength_long=np.array(wl_long),
                type_absorb=np.array(species, np.int32), n_band_absorb=nba, index_absorb=f(ia), i_band_k=f(ibk),
                i_scale_k=f(isk), i_scale_fnc=f(isf), k=f(k), w=f(w), scale=f(sc), p_ref=f(pr), t_ref=f(tr))


def _pade_sets(n_band, sw: bool, st: Stream):
    """Synthetic Pade coefficient sets (opt_prop_pade_2_mod.F90 form) for
    water droplets (re in m) and ice (De in m)."""
    drop = np.zeros((16, n_band, 1))
    ice = np.zeros((16, n_band, 1))
    for b in range(n_band):
        u = st.uniform((4,))
        # k_ext ~ 1.5/(rho_w re) per unit mass: c1/(1 + c4 re) with c4 re >> 1
        drop[0, b, 0] = 1.5e-3 * 1.0e7 * (0.9 + 0.2 * u[0])
        drop[3, b, 0] = 1.0e7
        ice[0, b, 0] = 1.0e-3 * 1.0e7 * (0.9 + 0.2 * u[1])
        ice[3, b, 0] = 1.0e7 / 3.0
        # co-albedo c7 + c8 re
        if sw:
            coalb = 1.0e-6 * 10.0 ** (3.0 * b / max(1, n_band - 1))
            drop[6, b, 0], drop[7, b, 0] = coalb, coalb * 2.0e4
            ice[6, b, 0], ice[7, b, 0] = 2.0 * coalb, coalb * 1.0e4
        else:
            drop[6, b, 0], drop[7, b, 0] = 0.3 + 0.3 * u[2], 5.0e3
            ice[6, b, 0], ice[7, b, 0] = 0.4 + 0.3 * u[3], 1.0e3
        # asymmetry c12 + c13 re
        drop[11, b, 0], drop[12, b, 0] = 0.80, 4.0e3
        ice[11, b, 0], ice[12, b, 0] = 0.72, 5.0e2
    return np.asfortranarray(drop), np.asfortranarray(ice)


def lw_spectrum(seed: int = 1, nk: int = 9, clouds: bool = False) -> Spectrum:
    """9 longwave bands, one absorber each, nk k-terms per band."""
    edges = np.array([10.0, 350.0, 500.0, 630.0, 820.0, 980.0, 1100.0, 1390.0, 1900.0, 3000.0])  # cm-1
    absorber = [1, 1, 1, 2, 1, 3, 1, 1, 1]        # H2O, CO2, O3 identifiers
    st = Stream(seed, 101)
    d = _base_spectrum(9, absorber, nk, st, 1.0e-2 / edges[1:], 1.0e-2 / edges[:-1])
    temps = np.linspace(150.0, 350.0, 81)
    t_ref = 250.0
    coeff = np.zeros((6, 9))
    for b in range(9):
        flux = _planck_band(edges[b], edges[b + 1], temps)
        coeff[:, b] = np.polynomial.polynomial.polyfit(temps / t_ref, flux, 5)
    sp = Spectrum(**d, n_deg_fit=5, t_ref_planck=t_ref, thermal_coeff=np.asfortranarray(coeff),
                  name=f"synthetic_lw_{nk}k_seed{seed}" + ("_cld" if clouds else ""))
    if clouds:
        sp.drop_parm_list, sp.ice_parm_list = _pade_sets(9, False, st)
        sp.i_drop_parm = np.array([5], np.int32)
        sp.i_ice_parm = np.array([20], np.int32)
    return sp


def sw_spectrum(seed: int = 2, nk: int = 8, clouds: bool = False) -> Spectrum:
    """6 shortwave bands, one absorber each, nk k-terms per band."""
    edges = np.array([0.2, 0.32, 0.5, 0.69, 1.19, 2.38, 10.0]) * 1.0e-6   # m
    absorber = [3, 3, 1, 1, 1, 2]
    st = Stream(seed, 102)
    d = _base_spectrum(6, absorber, nk, st, edges[:-1], edges[1:])
    # solar fractions from a 5778 K black body
    frac = np.zeros(6)
    for b in range(6):
        nu_lo, nu_hi = 1.0e-2 / edges[b + 1], 1.0e-2 / edges[b]
        frac[b] = _planck_band(nu_lo, nu_hi, [5778.0])[0]
    frac /= frac.sum()
    lam = np.sqrt(edges[:-1] * edges[1:]) / 1.0e-6
    ray = 8.6e-7 * lam ** -4.0
    sp = Spectrum(**d, solar_flux_band=frac, rayleigh_coeff=ray,
                  name=f"synthetic_sw_{nk}k_seed{seed}" + ("_cld" if clouds else ""))
    if clouds:
        sp.drop_parm_list, sp.ice_parm_list = _pade_sets(6, True, st)
        sp.i_drop_parm = np.array([5], np.int32)
        sp.i_ice_parm = np.array([20], np.int32)
    return sp


# ---------------------------------------------------------------------------
@dataclass
class Column:
    """Atmosphere, surface and optional aerosol/cloud fields in the
    reference's Fortran layouts (profile index fastest)."""
    n_profile: int
    n_layer: int
    p: np.ndarray
    t: np.ndarray
    p_level: np.ndarray
    t_level: np.ndarray
    mass: np.ndarray
    gas_mix_ratio: np.ndarray          # (n_profile, n_layer, n_species)
    z: np.ndarray                      # layer heights (m)
    t_ground: np.ndarray
    zen_0: np.ndarray | None = None
    solar_irrad: np.ndarray | None = None
    rho_alb: np.ndarray | None = None  # (n_profile, 2, n_band)
    aer: dict | None = None
    cld: dict | None = None
    density: np.ndarray | None = None  # (n_profile, n_layer) kg/m3, for continua
    extra: dict = field(default_factory=dict)


def atmosphere(n_profile: int, n_layer: int, species: np.ndarray, seed: int) -> Column:
    st = Stream(seed, 1)
    pl = np.logspace(1.0, 5.0, n_layer + 1)                   # level 0 = 10 Pa
    p_level = np.asfortranarray(np.broadcast_to(pl, (n_profile, n_layer + 1)))
    p = np.asfortranarray(np.sqrt(p_level[:, :-1] * p_level[:, 1:]))
    mass = np.asfortranarray((p_level[:, 1:] - p_level[:, :-1]) / GRAV)
    dT = (st.uniform((n_profile,)) * 2.0 - 1.0) * 10.0
    dq = 1.0 + 0.3 * (st.uniform((n_profile,)) * 2.0 - 1.0)

    def temp_of_z(z):
        return np.maximum(288.0 - 6.5e-3 * z, 217.0) + dT[:, None]

    # heights of levels, surface up (hypsometric, first order in each layer)
    zl = np.zeros((n_profile, n_layer + 1))
    for i in range(n_layer, 0, -1):
        tb = temp_of_z(zl[:, i:i + 1])[:, 0]
        zl[:, i - 1] = zl[:, i] + R_DRY * tb / GRAV * np.log(p_level[:, i] / p_level[:, i - 1])
    t_level = np.asfortranarray(temp_of_z(zl))
    z = np.asfortranarray(zl[:, 1:] + (zl[:, :-1] - zl[:, 1:]) * np.log(p_level[:, 1:] / p) / np.log(
        p_level[:, 1:] / p_level[:, :-1]))
    t = np.asfortranarray(temp_of_z(z))
    gas = np.zeros((n_profile, n_layer, len(species)), order="F")
    for j, s in enumerate(species):
        if s == 1:
            gas[:, :, j] = np.maximum(1.0e-2 * np.exp(-z / 2000.0), 3.0e-6) * dq[:, None]
        elif s == 2:
            gas[:, :, j] = 6.0e-4
        elif s == 3:
            gas[:, :, j] = 1.0e-5 * np.exp(-0.5 * np.log(p / 1000.0) ** 2)
        elif int(s) in TRACE_MMR:
            gas[:, :, j] = TRACE_MMR[int(s)]
    return Column(n_profile, n_layer, p, t, p_level, t_level, mass, gas, z,
                  t_ground=np.ascontiguousarray(t_level[:, -1]))


def add_density(col: Column, index_water: int) -> Column:
    """Moist air density of each layer (l_run_cdf.F90:1220-1235), which the
    water-vapour continuum needs; index_water is 1-based."""
    q = col.gas_mix_ratio[:, :, index_water - 1] if index_water > 0 else 0.0
    col.density = np.asfortranarray(col.p / (R_DRY * col.t * (1.0 + (28.966e-03 / 18.0153e-03 - 1.0) * q)))
    return col


def operational_case(sp: Spectrum, n_profile: int, n_layer: int, seed: int, solar: bool) -> Column:
    """Columns for an operational spectral file (many absorbers, continuum):
    the synthetic atmosphere with background amounts of the trace gases,
    its moist density and a surface for the source."""
    col = atmosphere(n_profile, n_layer, sp.type_absorb, seed)
    add_density(col, int(sp.index_water))
    if solar:
        add_sw_surface(col, sp.n_band, seed)
    else:
        add_lw_surface(col, sp.n_band)
    return col


def add_lw_surface(col: Column, n_band: int, emissivity: float = 0.98) -> Column:
    alb = np.zeros((col.n_profile, 2, n_band), order="F")
    alb[:, :, :] = 1.0 - emissivity
    col.rho_alb = alb
    return col


def add_sw_surface(col: Column, n_band: int, seed: int) -> Column:
    st = Stream(seed, 2)
    mu0 = 0.05 + 0.95 * st.uniform((col.n_profile,))
    alb = 0.05 + 0.35 * st.uniform((col.n_profile,))
    col.zen_0 = 1.0 / mu0
    col.solar_irrad = np.full(col.n_profile, SOLAR_CONSTANT)
    ra = np.zeros((col.n_profile, 2, n_band), order="F")
    ra[:, :, :] = alb[:, None, None]
    col.rho_alb = ra
    return col


def add_aerosol(col: Column, sp: Spectrum, seed: int) -> Column:
    st = Stream(seed, 3)
    n, L, nb = col.n_profile, col.n_layer, sp.n_band
    tau550 = np.exp(np.log(0.01) + (np.log(0.5) - np.log(0.01)) * st.uniform((n,)))
    om = 0.85 + 0.14 * st.uniform((n,))
    g = 0.6 + 0.15 * st.uniform((n,))
    k550 = 4.0e3
    low = col.z < 2000.0
    colmass = np.where(low, col.mass, 0.0).sum(axis=1)
    mmr = np.where(low, (tau550 / (k550 * np.maximum(colmass, 1e-12)))[:, None], 0.0)
    lam = np.sqrt(sp.wavelength_short * sp.wavelength_long) / 0.55e-6
    kext = k550 * lam ** -1.2                                            # (nb)
    shape = (n, L, 1, nb)
    ab = np.broadcast_to((kext[None, :] * (1.0 - om[:, None]))[:, None, None, :], shape)
    sc = np.broadcast_to((kext[None, :] * om[:, None])[:, None, None, :], shape)
    asy = np.broadcast_to(g[:, None, None, None], shape)
    col.aer = dict(n_mode=1, mode_mix_ratio=np.asfortranarray(mmr[:, :, None]),
                   mode_absorption=np.asfortranarray(ab), mode_scattering=np.asfortranarray(sc),
                   mode_asymmetry=np.asfortranarray(asy))
    return col


def add_aerosol_species(sp: Spectrum, seed: int, n_humidity: int = 11, n_phf: int = 2) -> Spectrum:
    """Classic aerosol species in the layout of spectral-file block 11
    (read_spectrum.F90:2335-2640): four species,
      1 water soluble (type 1), moist, humidities 0, 1/(n_humidity-1) .. 1
        (the equal spacing radiance_calc.F90:617-623 assumes), extinction
        growing with humidity;
      2 soot (type 4), dry;
      3 dust-like (type 2), dry with n_phf tabulated phase-function moments,
        the second not the square of the first;
      4 oceanic (type 3), moist with n_phf tabulated moments.
    Mass coefficients follow an Angstrom law in the band centre wavelength."""
    st = Stream(seed, 5)
    nb, nh, na = sp.n_band, n_humidity, 4
    lam = np.sqrt(sp.wavelength_short * sp.wavelength_long) / 0.55e-6     # (nb)
    hum = np.linspace(0.0, 1.0, nh)
    growth = 1.0 + 4.0 * hum ** 4                                         # (nh)
    k550 = np.array([4.0e3, 8.0e3, 1.0e3, 2.0e3])
    ang = np.array([1.4, 1.0, 0.3, 0.6])
    omega = np.array([0.95, 0.25, 0.9, 0.99]) - 0.04 * st.uniform((na,))
    g0 = np.array([0.65, 0.35, 0.72, 0.78]) + 0.05 * st.uniform((na,))
    abs_ = np.zeros((nh, na, nb), order="F")
    scat = np.zeros((nh, na, nb), order="F")
    phf = np.zeros((nh, n_phf, na, nb), order="F")
    moist = (True, False, False, True)
    n_terms = (1, 1, n_phf, n_phf)
    for j in range(na):
        ext = k550[j] * lam ** -ang[j]                                    # (nb)
        rows = growth if moist[j] else np.ones(nh)
        for h in range(nh):
            if not moist[j] and h > 0:
                continue
            w = min(omega[j] + (0.03 * hum[h] if moist[j] else 0.0), 0.999)
            abs_[h, j, :] = ext * rows[h] * (1.0 - w)
            scat[h, j, :] = ext * rows[h] * w
            g = np.minimum(g0[j] * (1.0 + 0.1 * hum[h] if moist[j] else 1.0) * lam ** -0.05, 0.9)
            for m in range(n_terms[j]):
                # tabulated moments of a phase function sharper than
                # Henyey-Greenstein beyond the first
                phf[h, m, j, :] = g ** (m + 1) * (1.0 if m == 0 else 1.08)
    sp.type_aerosol = np.array([1, 4, 2, 3], np.int32)
    sp.i_aerosol_parm = np.array([abi.IP_AEROSOL_PARAM_MOIST, abi.IP_AEROSOL_PARAM_DRY,
                                  abi.IP_AEROSOL_PARAM_PHF_DRY, abi.IP_AEROSOL_PARAM_PHF_MOIST], np.int32)
    sp.nhumidity = np.array([nh, 0, 0, nh], np.int32)
    sp.n_aerosol_phf_term = np.array(n_terms, np.int32)
    h2 = np.zeros((nh, na), order="F")
    h2[:, 0] = hum
    h2[:, 3] = hum
    sp.aerosol_humidities = h2
    sp.aerosol_abs, sp.aerosol_scat, sp.aerosol_phf = abs_, scat, phf
    sp.name = f"{sp.name}_aer{seed}_{nh}h_{n_phf}m"
    return sp


def add_aerosol_mix(col: Column, seed: int, entries=(1, 2, 3, 4), sources=None, tau550: float = 0.3) -> Column:
    """Mixing ratios of classic aerosol entries (def_aer.F90:26-34) for the
    species of add_aerosol_species: entry e refers to species entries[e]
    (1-based, repeats allowed) with source sources[e] (IP_AERSRC_*;
    classic_ron by default), each in the lowest 3 km with a column loading
    near tau550/len(entries)/k550, and the mean relative humidity of each
    layer in [0, 1], exactly 0 and exactly 1 included."""
    st = Stream(seed, 6)
    n, L, ne = col.n_profile, col.n_layer, len(entries)
    low = col.z < 3000.0
    colmass = np.maximum(np.where(low, col.mass, 0.0).sum(axis=1), 1e-12)
    mr = np.zeros((n, L, ne), order="F")
    for e in range(ne):
        scale = (0.2 + 1.6 * st.uniform((n,))) * tau550 / ne / 4.0e3
        prof = np.exp(-col.z / 1500.0) * (0.5 + st.uniform((n, L)))
        mr[:, :, e] = np.where(low, (scale / colmass)[:, None] * prof, 0.0)
    rh = np.asfortranarray(np.clip(st.uniform((n, L)) * 1.1 - 0.05, 0.0, 1.0))
    col.aer = dict(col.aer or {})
    col.aer.update(mix_ratio=mr, mr_type_index=np.asarray(entries, np.int32),
                   mr_source=np.asarray(sources if sources is not None else [abi.IP_AERSRC_CLASSIC_RON] * ne,
                                        np.int32),
                   mean_rel_humidity=rh)
    return col


def add_prescribed_aerosol(sp: Spectrum, col: Column, seed: int, species=(2,), n_level: int = 30,
                           n_phf: int = 2, p_top: float = 5.0e3) -> tuple[Spectrum, Column]:
    """Prescribed optical properties (l_run_cdf's overlay of observations,
    def_aer.F90:46-60) for the given 1-based species of add_aerosol_species,
    which become unparametrized in a copy of the spectrum: per column,
    n_level pressures log-spaced from p_top to just above the surface (layers
    above p_top lie outside the levels), volume absorption and scattering
    [1/m] decaying with height, and n_phf phase-function moments.  Returns
    (spectrum, column); col.aer gains the *_prsc arrays."""
    import copy
    st = Stream(seed, 7)
    sp2 = copy.copy(sp)
    parm = np.array(sp.i_aerosol_parm, np.int32)
    nsp, nb, n = len(parm), sp.n_band, col.n_profile
    lam = np.sqrt(sp.wavelength_short * sp.wavelength_long) / 0.55e-6
    pl = np.zeros((n, n_level, nsp), order="F")
    ab = np.zeros((n, n_level, nsp, nb), order="F")
    sc = np.zeros((n, n_level, nsp, nb), order="F")
    ph = np.zeros((n, n_level, n_phf, nsp, nb), order="F")
    nlev = np.ones(nsp, np.int32)
    nmom = np.ones(nsp, np.int32)
    for s in species:
        j = s - 1
        parm[j] = abi.IP_AEROSOL_UNPARAMETRIZED
        nlev[j], nmom[j] = n_level, n_phf
        p_bot = col.p_level[:, -1] * (0.995 - 0.01 * st.uniform((n,)))
        lev = np.exp(np.linspace(0.0, 1.0, n_level)[None, :] * np.log(p_bot / p_top)[:, None]) * p_top
        pl[:, :, j] = lev
        ext0 = 2.0e-5 * (0.5 + st.uniform((n,)))                          # 1/m at the surface
        shape = (lev / p_bot[:, None]) ** 6                                 # ~ 1.3 km scale height
        w = 0.8 + 0.15 * st.uniform((n,))
        for b in range(nb):
            e = ext0[:, None] * shape * lam[b] ** -0.5
            ab[:, :, j, b] = e * (1.0 - w[:, None])
            sc[:, :, j, b] = e * w[:, None]
            g = 0.6 + 0.1 * (lev / p_bot[:, None])
            for m in range(n_phf):
                ph[:, :, m, j, b] = g ** (m + 1) * (1.0 if m == 0 else 1.05)
    sp2.i_aerosol_parm = parm
    sp2.name = f"{sp.name}_prsc{''.join(map(str, species))}"
    col.aer = dict(col.aer or {})
    col.aer.update(n_opt_level_prsc=nlev, n_phase_term_prsc=nmom, pressure_prsc=pl, absorption_prsc=ab,
                   scattering_prsc=sc, phase_fnc_prsc=ph)
    return sp2, col


def add_clouds(col: Column, seed: int, n_subcol: int = 16, decorrelation_m: float = 2000.0,
               cloud_prob: float = 0.3, p_top: float = 1.0e4) -> Column:
    """Cloud fields as set_cld leaves them for ip_cloud_ice_water
    (socrates_set_cld.F90:500-530, 800-845): normalised phase fractions and
    in-cloud mixing ratios; overlap decorrelation in pressure from the local
    scale height (dp = p g dz / (R T)).  Cloud is confined to the
    troposphere (layer pressure above p_top, 100 hPa by default)."""
    st = Stream(seed, 4)
    n, L = col.n_profile, col.n_layer
    cloudy = (st.uniform((n, L)) < cloud_prob) & (col.p > p_top)
    frac = np.where(cloudy, st.uniform((n, L)), 0.0)
    rho = col.p / (R_DRY * col.t)
    liquid = col.z < 6000.0
    nrm = np.sqrt(-2.0 * np.log(np.maximum(st.uniform((n, L)), 1e-300))) * np.cos(2 * np.pi * st.uniform((n, L)))
    lwc = 0.1e-3 * np.exp(1.0 * nrm)
    iwc = 0.02e-3 * np.exp(1.0 * nrm)
    re = (4.0 + 12.0 * st.uniform((n, L))) * 1e-6
    de = (20.0 + 100.0 * st.uniform((n, L))) * 1e-6
    liq_mmr = np.where(cloudy & liquid, lwc / rho, 0.0)
    ice_mmr = np.where(cloudy & ~liquid, iwc / rho, 0.0)
    w_cloud = np.where(frac > 0.0, frac, 0.0)
    fw = np.where((frac > 0) & liquid, 1.0, 0.0)
    fi = np.where((frac > 0) & ~liquid, 1.0, 0.0)
    f = np.asfortranarray
    cond = f(np.stack([liq_mmr, ice_mmr], axis=2))
    dim = f(np.stack([re, de], axis=2))
    dp_corr = col.p * GRAV * decorrelation_m / (R_DRY * col.t)
    seeds = (st.uniform((n,)) * 2.0e9).astype(np.int32) + 1
    col.cld = dict(w_cloud=f(w_cloud), frac_cloud=f(np.stack([fw, fi], axis=2)),
                   condensed_mix_ratio=cond, condensed_dim_char=dim,
                   dp_corr_cloud=f(dp_corr), dp_corr_cond=f(0.5 * dp_corr), rand_seed=seeds, n_subcol_gen=n_subcol)
    return col


def window(col: Column, start: int, n: int, alloc=None) -> Column:
    """Columns start .. start+n-1 of col as a new Column (copies, Fortran
    order).  Per-column arrays are those whose first extent is n_profile.
    `alloc(shape, dtype)`, when given, provides the destination arrays
    (e.g. in page-locked memory)."""
    import copy
    c = copy.copy(col)
    c.n_profile = n
    sl = slice(start, start + n)

    def cut(v):
        if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == col.n_profile:
            if alloc is None:
                return np.asfortranarray(v[sl])
            out = alloc(v[sl].shape, v.dtype)
            out[...] = v[sl]
            return out
        return v

    for name in ("p", "t", "p_level", "t_level", "mass", "gas_mix_ratio", "z", "t_ground", "zen_0", "solar_irrad",
                 "rho_alb", "density"):
        setattr(c, name, cut(getattr(col, name)))
    if col.aer:
        c.aer = {k: cut(v) for k, v in col.aer.items()}
    if col.cld:
        c.cld = {k: cut(v) for k, v in col.cld.items()}
    return c


# ---------------------------------------------------------------------------
def config1(n_profile: int = 1000, n_layer: int = 60, seed: int = 1):
    """Plain longwave clear sky, no scattering (Elsasser 1.66)."""
    sp = lw_spectrum(seed, 9)
    col = atmosphere(n_profile, n_layer, sp.type_absorb, seed)
    add_lw_surface(col, sp.n_band)
    return sp, col


def config2(n_profile: int = 10000, n_layer: int = 100, seed: int = 2):
    """Shortwave PIFM80, delta-Eddington rescaling, Rayleigh and aerosol."""
    sp = sw_spectrum(seed, 8)
    col = atmosphere(n_profile, n_layer, sp.type_absorb, seed)
    add_sw_surface(col, sp.n_band, seed)
    add_aerosol(col, sp, seed)
    return sp, col


def config3(n_profile: int = 65536, n_layer: int = 85, seed: int = 3, n_subcol: int = 16):
    """All-sky LW + SW with McICA clouds (exponential-random overlap)."""
    lw = lw_spectrum(seed, 9, clouds=True)
    sw = sw_spectrum(seed, 8, clouds=True)
    species = np.array(sorted(set(lw.type_absorb) | set(sw.type_absorb)), np.int32)
    col = atmosphere(n_profile, n_layer, species, seed)
    add_clouds(col, seed, n_subcol)
    return lw, sw, col
