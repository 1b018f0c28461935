"""Spectral files: the host-side model of the reference's StrSpecData.

``Spectrum`` holds the arrays of src/radiance_core/def_spectrum.F90 as
Fortran-ordered numpy arrays with the same 1-based meaning (stored 0-based),
``write_text``/``read_text`` handle the reference's text ``*BLOCK`` format
for the blocks the two-stream path uses (0 summary, 1 band limits, 2 solar
spectrum, 3 Rayleigh, 4 absorbers per band, 5 k-terms, 6 Planck polynomial,
10 droplets, 12 ice; layouts of read_spectrum.F90:557-1214), and
``to_desc`` produces the flat ``socgpu_spectrum_desc`` of the C-ABI.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

from pathlib import Path

import numpy as np

from . import abi

GAS_NAMES = {1: "Water Vapour", 2: "Carbon Dioxide", 3: "Ozone", 4: "Dinitrogen Oxide", 5: "Carbon monoxide",
             6: "Methane", 7: "Oxygen"}


# Parameters of each scaling function (rad_pcf.F90 n_scale_variable).
N_SCALE_VARIABLE = {0: 0, 1: 2, 2: 3, 3: 4, 4: 0, 5: 0, 6: 6, 7: 8, 8: 10, 9: 0, 10: 0}


# Molar weights [g/mol] of the absorbers by gas identifier (the published
# values of J. A. Duffy, General Inorganic Chemistry (1970), and NIST, as
# gas_list_pcf.F90:303-330 lists them); used for self-broadened gas fractions.
MOLAR_WEIGHT = {1: 18.0153, 2: 44.0100, 3: 47.9982, 4: 44.0128, 5: 28.0106, 6: 16.0430, 7: 31.9988, 8: 30.0061,
                9: 64.0628, 10: 46.0055, 11: 17.0306, 12: 63.0129, 13: 28.0134, 14: 137.3686, 15: 120.9140,
                16: 187.3765, 17: 86.46892, 18: 120.02227, 19: 102.03184, 20: 170.921, 21: 63.866, 22: 66.9409,
                23: 2.01588, 24: 4.002602, 25: 60.075}


def _f(a, dtype):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


def _fields13(line):
    """The 1PE13.6 fields of one record."""
    line = line.rstrip()
    return [float(line[i:i + 13]) for i in range(0, len(line), 13) if line[i:i + 13].strip()]


def read_wenyi_tables(path) -> dict:
    """The CO2 (band 4) and O3 (band 6) tables of ip_scale_wenyi from their
    data file (socrates_gb300.wenyi: the reference compiles the tables into
    its source; the converter there writes them out once as data)."""
    from socrates_gb300 import wenyi
    return wenyi.read_data(path)


def _read_k_file(path, n_band, n_abs, nd_k, recs, ia, nba, isb, n_pre, n_tmp):
    """Lookup tables of the '_k' file in the order read_spectrum.F90:1420-1560
    reads them: the P/T grid, the gas fractions of self-broadened absorbers,
    one table per (band, absorber) record of block 5, then the
    temperature-only tables."""
    text = Path(path).read_text().splitlines()

    def values(q, n):
        out = []
        while len(out) < n:
            out += _fields13(text[q])
            q += 1
        return out[:n], q

    def block(title):
        for q, ln in enumerate(text):
            if ln.startswith("*BLOCK") and ln[8:8 + len(title)] == title:
                return q
        raise ValueError(f"{path}: no '{title}' block")

    out = {}
    if any(r[4] == abi.IP_SCALE_LOOKUP for r in recs):
        q = block("k-table") + 3
        p_lk = np.zeros(n_pre)
        t_lk = np.zeros((n_tmp, n_pre))
        for ip in range(n_pre):
            v, q = values(q, 1 + n_tmp)
            p_lk[ip] = np.log(v[0])
            t_lk[:, ip] = v[1:]
        sb = isb is not None and bool(np.any(isb > 0))
        gf = None
        if sb:
            n_gf = int(text[q + 1][14:18])
            gf, q = values(q + 2, n_gf)
            gf = np.array(gf)
            nsb = int(isb.max())
            k_sb = np.zeros((n_tmp, n_pre, n_gf, nd_k, nsb, n_band))
        k_lk = np.zeros((n_tmp, n_pre, nd_k, n_abs, n_band))
        for b, g, nk, sk, fnc, *_ in recs:
            if fnc != abi.IP_SCALE_LOOKUP:
                continue
            q += 2
            if sb and isb[g] > 0:
                for t in range(nk):
                    for ig in range(n_gf):
                        for ip in range(n_pre):
                            v, q = values(q, n_tmp)
                            k_sb[:, ip, ig, t, isb[g] - 1, b] = v
            else:
                for t in range(nk):
                    for ip in range(n_pre):
                        v, q = values(q, n_tmp)
                        k_lk[:, ip, t, g, b] = v
        out.update(p_lookup=p_lk, t_lookup=_f(t_lk, np.float64), k_lookup=_f(k_lk, np.float64))
        if sb:
            out.update(index_sb=isb, gf_lookup=gf, k_lookup_sb=_f(k_sb, np.float64))
    t_gases = sorted({r[1] for r in recs if r[4] == abi.IP_SCALE_T_LOOKUP})
    if t_gases:
        q = block("temperature k-tables")
        ndt = int(text[q + 2][9:13])
        q += 3
        n_t = np.zeros(n_abs, np.int32)
        t_g = np.zeros((ndt, n_abs))
        for g in t_gases:
            n_t[g] = int(text[q + 1][27:31])
            v, q = values(q + 2, n_t[g])
            t_g[: n_t[g], g] = v
        fnc_of = {(r[0], r[1]): r[4] for r in recs}
        nk_of = {(r[0], r[1]): r[2] for r in recs}
        k_t = np.zeros((ndt, nd_k, n_abs, n_band))
        for b in range(n_band):
            for j in range(int(nba[b])):
                g = int(ia[j, b]) - 1
                if fnc_of.get((b, g)) != abi.IP_SCALE_T_LOOKUP:
                    continue
                q += 2
                for t in range(nk_of[(b, g)]):
                    v, q = values(q, n_t[g])
                    k_t[: n_t[g], t, g, b] = v
        out.update(n_t_lookup_gas=n_t, t_lookup_gas=_f(t_g, np.float64), k_t_lookup_gas=_f(k_t, np.float64))
    return out


@dataclass
class Spectrum:
    """Arrays of StrSpecData needed by the two-stream path (0-based storage)."""
    n_band: int
    wavelength_short: np.ndarray            # (n_band) m
    wavelength_long: np.ndarray
    type_absorb: np.ndarray                 # (n_absorb) gas identifiers
    n_band_absorb: np.ndarray               # (n_band)
    index_absorb: np.ndarray                # (nd_species, n_band) 1-based species, 0 unused
    i_band_k: np.ndarray                    # (n_band, n_absorb)
    i_scale_k: np.ndarray                   # (n_band, n_absorb)
    i_scale_fnc: np.ndarray                 # (n_band, n_absorb)
    k: np.ndarray                           # (nd_k_term, n_band, n_absorb)
    w: np.ndarray                           # (nd_k_term, n_band, n_absorb)
    scale: np.ndarray                       # (nd_scale_variable, nd_k_term, n_band, n_absorb)
    p_ref: np.ndarray                       # (n_absorb, n_band)
    t_ref: np.ndarray                       # (n_absorb, n_band)
    solar_flux_band: np.ndarray | None = None
    rayleigh_coeff: np.ndarray | None = None
    n_deg_fit: int = 0
    t_ref_planck: float = 0.0
    thermal_coeff: np.ndarray | None = None  # (n_deg_fit+1, n_band)
    # blocks 10 and 12: cloud parameter sets, indexed by the file's type number
    drop_parm_list: np.ndarray | None = None # (n_parameter, n_band, n_drop_type)
    i_drop_parm: np.ndarray | None = None    # (n_drop_type) scheme, 0 where the type is undefined
    ice_parm_list: np.ndarray | None = None  # (n_parameter, n_band, n_ice_type)
    i_ice_parm: np.ndarray | None = None
    drop_n_parm: np.ndarray | None = None    # (n_drop_type) coefficients the file gives per band
    drop_n_phf: np.ndarray | None = None     # (n_drop_type) phase-function moments
    drop_parm_min_dim: np.ndarray | None = None  # (n_drop_type) range of validity [m]
    drop_parm_max_dim: np.ndarray | None = None
    ice_n_parm: np.ndarray | None = None
    ice_n_phf: np.ndarray | None = None
    ice_parm_min_dim: np.ndarray | None = None
    ice_parm_max_dim: np.ndarray | None = None
    # block 13: Doppler broadening (per absorber)
    l_doppler: np.ndarray | None = None      # (n_absorb) 0/1
    doppler_cor: np.ndarray | None = None    # (n_absorb)
    # blocks 8 and 9: continua (StrSpecCont)
    n_band_continuum: np.ndarray | None = None   # (n_band)
    index_continuum: np.ndarray | None = None    # (n_band, nd_continuum) 1 self, 2 foreign
    index_water: int = 0                         # 1-based absorber index of water vapour
    i_scale_fnc_cont: np.ndarray | None = None   # (n_band, nd_continuum)
    k_cont: np.ndarray | None = None             # (n_band, nd_continuum) m5/(kg mol)
    scale_cont: np.ndarray | None = None         # (nd_scale_variable, n_band, nd_continuum)
    p_ref_cont: np.ndarray | None = None         # (nd_continuum, n_band)
    t_ref_cont: np.ndarray | None = None         # (nd_continuum, n_band)
    i_overlap: np.ndarray | None = None          # (n_band) overlap method of each band (block 4 version 1)
    # lookup-table k scaling: block 5 with the '_k' companion file
    p_lookup: np.ndarray | None = None           # (n_pre) ln(p / Pa)
    t_lookup: np.ndarray | None = None           # (n_tmp, n_pre) K
    k_lookup: np.ndarray | None = None           # (n_tmp, n_pre, nd_k_term, n_absorb, n_band)
    index_sb: np.ndarray | None = None           # (n_absorb) 1-based self-broadened index, 0 none
    gf_lookup: np.ndarray | None = None          # (n_gas_frac)
    k_lookup_sb: np.ndarray | None = None        # (n_tmp, n_pre, n_gas_frac, nd_k_term, nd_species_sb, n_band)
    n_t_lookup_gas: np.ndarray | None = None     # (n_absorb)
    t_lookup_gas: np.ndarray | None = None       # (nd_t_lookup_gas, n_absorb) K
    k_t_lookup_gas: np.ndarray | None = None     # (nd_t_lookup_gas, nd_k_term, n_absorb, n_band)
    # CO2 and O3 tables of ip_scale_wenyi (the reference compiles them in)
    wenyi_plg: np.ndarray | None = None          # (26)
    wenyi_ttb: np.ndarray | None = None          # (10)
    wenyi_tto: np.ndarray | None = None          # (9)
    wenyi_gk250b: np.ndarray | None = None       # (n_term4)
    wenyi_gk4: np.ndarray | None = None          # (10, 26, n_term4)
    wenyi_gk6: np.ndarray | None = None          # (9, 26, n_term6)
    # block 11: classic aerosol species (StrSpecAerosol, read_spectrum.F90:2335-2640)
    type_aerosol: np.ndarray | None = None       # (n_aerosol) type numbers
    i_aerosol_parm: np.ndarray | None = None     # (n_aerosol) IP_AEROSOL_PARAM_*
    nhumidity: np.ndarray | None = None          # (n_aerosol) 0 for dry species
    n_aerosol_phf_term: np.ndarray | None = None # (n_aerosol)
    aerosol_humidities: np.ndarray | None = None # (nd_humidity, n_aerosol)
    aerosol_abs: np.ndarray | None = None        # (nd_humidity, n_aerosol, n_band) m2/kg
    aerosol_scat: np.ndarray | None = None       # (nd_humidity, n_aerosol, n_band) m2/kg
    aerosol_phf: np.ndarray | None = None        # (nd_humidity, nd_phase_term, n_aerosol, n_band)
    name: str = "spectrum"
    _keep: list = field(default_factory=list, repr=False)

    @property
    def n_absorb(self) -> int:
        return int(self.type_absorb.size)

    @property
    def nd_k_term(self) -> int:
        return int(self.k.shape[0])

    @property
    def n_gpoint(self) -> int:
        """Number of k-term products over all bands (random overlap)."""
        total = 0
        for b in range(self.n_band):
            n = 1
            for j in range(int(self.n_band_absorb[b])):
                g = int(self.index_absorb[j, b]) - 1
                n *= int(self.i_band_k[b, g])
            total += n
        return total

    def gpoint_bands(self) -> np.ndarray:
        out = []
        for b in range(self.n_band):
            n = 1
            for j in range(int(self.n_band_absorb[b])):
                n *= int(self.i_band_k[b, int(self.index_absorb[j, b]) - 1])
            out += [b] * n
        return np.array(out, dtype=np.int32)

    # ------------------------------------------------------------------
    def to_desc(self) -> abi.SpectrumDesc:
        """Flat C view; the arrays are kept alive on the Spectrum."""
        keep = []

        def dp(a):
            if a is None:
                return None
            a = _f(a, np.float64)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_double))

        def ip(a):
            if a is None:
                return None
            a = _f(a, np.int32)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_int))

        d = abi.SpectrumDesc()
        d.nd_band = self.n_band
        d.nd_species = max(1, self.index_absorb.shape[0])
        d.nd_k_term = self.nd_k_term
        d.nd_scale_variable = self.scale.shape[0]
        d.n_band = self.n_band
        d.wavelength_short = dp(self.wavelength_short)
        d.wavelength_long = dp(self.wavelength_long)
        d.solar_flux_band = dp(self.solar_flux_band)
        d.i_rayleigh_scheme = abi.IP_RAYLEIGH_TOTAL
        d.rayleigh_coeff = dp(self.rayleigh_coeff)
        d.n_absorb = self.n_absorb
        d.type_absorb = ip(self.type_absorb)
        d.n_band_absorb = ip(self.n_band_absorb)
        if self.i_overlap is not None:
            d.i_overlap = ip(self.i_overlap)
        # index_absorb is (nd_species, n_band); nd_species also indexes p_ref/t_ref
        nds = d.nd_species
        ia = np.zeros((nds, self.n_band), np.int32)
        ia[: self.index_absorb.shape[0]] = self.index_absorb
        d.index_absorb = ip(ia)
        d.i_band_k = ip(self.i_band_k)
        d.i_scale_k = ip(self.i_scale_k)
        d.i_scale_fnc = ip(self.i_scale_fnc)
        d.k = dp(self.k)
        d.w = dp(self.w)
        d.scale = dp(self.scale)
        pr = np.zeros((nds, self.n_band))
        tr = np.zeros((nds, self.n_band))
        pr[: self.n_absorb] = self.p_ref
        tr[: self.n_absorb] = self.t_ref
        d.p_ref = dp(pr)
        d.t_ref = dp(tr)
        d.l_doppler = ip(self.l_doppler) if self.l_doppler is not None else None
        d.doppler_cor = dp(self.doppler_cor) if self.doppler_cor is not None else None
        if self.n_band_continuum is not None:
            ndc = self.index_continuum.shape[1]
            d.nd_continuum = ndc
            d.n_band_continuum = ip(self.n_band_continuum)
            d.index_continuum = ip(self.index_continuum)
            d.index_water = int(self.index_water)
            d.i_scale_fnc_cont = ip(self.i_scale_fnc_cont)
            d.k_cont = dp(self.k_cont)
            nsv = self.scale_cont.shape[0]
            if nsv != d.nd_scale_variable:
                sc = np.zeros((d.nd_scale_variable, self.n_band, ndc))
                m = min(nsv, d.nd_scale_variable)
                sc[:m] = self.scale_cont[:m]
                d.scale_cont = dp(sc)
            else:
                d.scale_cont = dp(self.scale_cont)
            d.p_ref_cont = dp(self.p_ref_cont)
            d.t_ref_cont = dp(self.t_ref_cont)
        nk = self.nd_k_term
        if self.k_lookup is not None:
            n_tmp, n_pre = self.t_lookup.shape
            d.n_tmp, d.n_pre = n_tmp, n_pre
            d.p_lookup = dp(self.p_lookup)
            d.t_lookup = dp(self.t_lookup)
            kl = np.zeros((n_tmp, n_pre, nk, nds, self.n_band))
            kl[:, :, :, : self.n_absorb] = self.k_lookup
            d.k_lookup = dp(kl)
        if self.index_sb is not None and self.k_lookup_sb is not None:
            isb = np.zeros(nds, np.int32)
            isb[: self.n_absorb] = self.index_sb
            d.index_sb = ip(isb)
            d.nd_species_sb = int(self.k_lookup_sb.shape[4])
            d.n_gas_frac = int(self.gf_lookup.size)
            d.gf_lookup = dp(self.gf_lookup)
            d.k_lookup_sb = dp(self.k_lookup_sb)
        mw = np.zeros(nds)
        mw[: self.n_absorb] = [MOLAR_WEIGHT.get(int(t), 0.0) for t in self.type_absorb]
        d.molar_weight = dp(mw)
        if self.k_t_lookup_gas is not None:
            ndt = int(self.t_lookup_gas.shape[0])
            d.nd_t_lookup_gas = ndt
            nt = np.zeros(nds, np.int32)
            nt[: self.n_absorb] = self.n_t_lookup_gas
            d.n_t_lookup_gas = ip(nt)
            tg = np.zeros((ndt, nds))
            tg[:, : self.n_absorb] = self.t_lookup_gas
            d.t_lookup_gas = dp(tg)
            kt = np.zeros((ndt, nk, nds, self.n_band))
            kt[:, :, : self.n_absorb] = self.k_t_lookup_gas
            d.k_t_lookup_gas = dp(kt)
        if self.wenyi_plg is not None:
            d.wenyi_plg = dp(self.wenyi_plg)
            d.wenyi_ttb = dp(self.wenyi_ttb)
            d.wenyi_tto = dp(self.wenyi_tto)
            d.wenyi_gk250b = dp(self.wenyi_gk250b)
            d.wenyi_gk4 = dp(self.wenyi_gk4)
            d.wenyi_gk6 = dp(self.wenyi_gk6)
            d.wenyi_n_term4 = int(self.wenyi_gk4.shape[2])
            d.wenyi_n_term6 = int(self.wenyi_gk6.shape[2])
        if self.thermal_coeff is not None:
            d.n_deg_fit = self.n_deg_fit
            d.t_ref_planck = self.t_ref_planck
            d.nd_thermal_coeff = self.thermal_coeff.shape[0]
            d.thermal_coeff = dp(self.thermal_coeff)
        # both lists share nd_cloud_parameter (StrSpecDim), so pad the shorter
        ncp = max([a.shape[0] for a in (self.drop_parm_list, self.ice_parm_list) if a is not None], default=0)
        pad = lambda a: np.asfortranarray(np.concatenate(
            [a, np.zeros((ncp - a.shape[0],) + a.shape[1:])], axis=0)) if a.shape[0] < ncp else a
        if self.drop_parm_list is not None:
            d.nd_cloud_parameter = ncp
            d.nd_drop_type = self.drop_parm_list.shape[2]
            d.drop_parm_list = dp(pad(self.drop_parm_list))
            d.i_drop_parm = ip(self.i_drop_parm)
            d.l_drop_type = ip((np.asarray(self.i_drop_parm) > 0).astype(np.int32))
            if self.drop_parm_min_dim is not None and self.drop_parm_max_dim is not None:
                d.drop_parm_min_dim, d.drop_parm_max_dim = dp(self.drop_parm_min_dim), dp(self.drop_parm_max_dim)
        if self.ice_parm_list is not None:
            d.nd_cloud_parameter = ncp
            d.nd_ice_type = self.ice_parm_list.shape[2]
            d.ice_parm_list = dp(pad(self.ice_parm_list))
            d.i_ice_parm = ip(self.i_ice_parm)
            d.l_ice_type = ip((np.asarray(self.i_ice_parm) > 0).astype(np.int32))
            if self.ice_parm_min_dim is not None and self.ice_parm_max_dim is not None:
                d.ice_parm_min_dim, d.ice_parm_max_dim = dp(self.ice_parm_min_dim), dp(self.ice_parm_max_dim)
        if self.aerosol_abs is not None:
            d.n_aerosol = d.nd_aerosol_species = int(self.aerosol_abs.shape[1])
            d.nd_humidity = int(self.aerosol_abs.shape[0])
            d.nd_phase_term = int(self.aerosol_phf.shape[1])
            d.type_aerosol = ip(self.type_aerosol)
            d.i_aerosol_parm = ip(self.i_aerosol_parm)
            d.nhumidity = ip(self.nhumidity)
            d.n_aerosol_phf_term = ip(self.n_aerosol_phf_term)
            d.aerosol_humidities = dp(self.aerosol_humidities)
            d.aerosol_abs = dp(self.aerosol_abs)
            d.aerosol_scat = dp(self.aerosol_scat)
            d.aerosol_phf = dp(self.aerosol_phf)
        self._keep = keep
        return d

    # ------------------------------------------------------------------
    def save_npz(self, path) -> None:
        """Store the arrays (for fixtures of parsed spectral files)."""
        from dataclasses import fields
        out = {}
        for f in fields(self):
            if f.name.startswith("_"):
                continue
            v = getattr(self, f.name)
            if v is None:
                continue
            out[f.name] = np.asarray(v)
        np.savez_compressed(path, **out)

    @classmethod
    def load_npz(cls, path, prefix: str = "") -> "Spectrum":
        from dataclasses import fields
        data = np.load(path)
        kw = {}
        for f in fields(cls):
            key = prefix + f.name
            if key not in data.files:
                continue
            v = data[key]
            if v.ndim == 0:
                v = v.item()
            elif v.dtype.kind in "fi":
                v = np.asfortranarray(v)
            kw[f.name] = v
        return cls(**kw)

    # ------------------------------------------------------------------
    def write_text(self, path) -> None:
        """Write the spectral file in the reference's text block format."""
        L = []
        e = lambda x: f"{x:16.9E}"
        L.append("*BLOCK: TYPE =    0: SUBTYPE =    0: VERSION =    2")
        L.append("Summary of spectral data.")
        L.append(f"Number of spectral bands = {self.n_band:5d}")
        L.append(f"Total number of gaseous absorbers = {self.n_absorb:5d}")
        L.append(f"Maximum number of k-terms in a band = {self.nd_k_term:5d}")
        n_aer = 0 if self.aerosol_abs is None else int(self.aerosol_abs.shape[1])
        L.append(f"Total number of aerosols = {n_aer:5d}")
        L.append("List of indexing numbers and absorbers.")
        L.append("Index       Absorber(identifier and name)")
        for i, t in enumerate(self.type_absorb):
            L.append(f"{i + 1:5d}       {int(t):5d}       {GAS_NAMES.get(int(t), 'Gas'):20s}")
        L.append("List of indexing numbers of aerosols.")
        L.append("Index       Aerosol(type number and name)")
        for i in range(n_aer):
            L.append(f"{i + 1:5d}       {int(self.type_aerosol[i]):5d}       {'Aerosol':20s}")
        L.append("*END")
        L.append("*BLOCK: TYPE =    1: SUBTYPE =    0: VERSION =    0")
        L.append("Specification of spectral intervals")
        L.append("Limits of spectral intervals (wavelengths in m.)")
        L.append("Band        Lower limit         Upper limit")
        for b in range(self.n_band):
            L.append(f"{b + 1:5d}       {e(self.wavelength_short[b])}    {e(self.wavelength_long[b])}")
        L.append("*END")
        if self.solar_flux_band is not None:
            L.append("*BLOCK: TYPE =    2: SUBTYPE =    0: VERSION =    0")
            L.append("Normalized solar flux in each spectral interval.")
            L.append("Band        Fraction of incident solar flux")
            for b in range(self.n_band):
                L.append(f"{b + 1:5d}       {e(self.solar_flux_band[b])}")
            L.append("*END")
        if self.rayleigh_coeff is not None:
            L.append("*BLOCK: TYPE =    3: SUBTYPE =    0: VERSION =    0")
            # three header records: read_spectrum.F90:882 skips them with '(//)'
            L.append("Rayleigh mass scattering coefficients at STP: unit m**2/kg")
            L.append("Band        Rayleigh coefficient")
            L.append("                 m2/kg")
            for b in range(self.n_band):
                L.append(f"{b + 1:5d}       {e(self.rayleigh_coeff[b])}")
            L.append("*END")
        v4 = self.i_overlap is not None
        L.append(f"*BLOCK: TYPE =    4: SUBTYPE =    0: VERSION =    {1 if v4 else 0}")
        L.append("Gaseous absorbers in each interval")
        L.append("(The number is the indexing number of the species as set out")
        L.append(" in the summary block 0.)")
        L.append("A zero indicates that there in no gaseous absorption in the interval.")
        L.append("Band, number of absorbers and overlap method, followed by indexing numbers" if v4 else
                 "Band        Number of active absorbers followed by indexing numbers")
        for b in range(self.n_band):
            L.append(f"{b + 1:5d}       {int(self.n_band_absorb[b]):5d}"
                     + (f"       {int(self.i_overlap[b]):5d}" if v4 else ""))
            if self.n_band_absorb[b] > 0:
                L.append("   " + "".join(f"{int(self.index_absorb[j, b]):5d}" for j in range(int(self.n_band_absorb[b]))))
        L.append("*END")
        tables = self.k_lookup is not None or self.k_t_lookup_gas is not None
        L.append(f"*BLOCK: TYPE =    5: SUBTYPE =    0: VERSION =    {1 if tables else 0}")
        L.append("Exponential sum fiting coefficients: (exponents: m2/kg)")
        if self.index_sb is not None and self.k_lookup_sb is not None:
            # read_spectrum.F90 block 5_0_1: (/,6(2x, i3))
            L.append("Self-broadened indexing numbers of all absorbers.")
            L.append("(Zero means no self-broadening.)")
            isb = [int(x) for x in self.index_sb]
            for q in range(0, len(isb), 6):
                L.append("".join(f"  {x:3d}" for x in isb[q:q + 6]))
        L.append("Band        Gas, Number of k-terms, Scaling type and scaling function,")
        L.append("             followed by reference pressure and temperature,")
        L.append("                   k-terms, weights and scaling parameters.")
        for b in range(self.n_band):
            for j in range(int(self.n_band_absorb[b])):
                g = int(self.index_absorb[j, b]) - 1
                nk = int(self.i_band_k[b, g])
                fnc = int(self.i_scale_fnc[b, g])
                L.append(f"{b + 1:5d}       {g + 1:5d}       {nk:5d}       {int(self.i_scale_k[b, g]):5d}       {fnc:5d}")
                if fnc == abi.IP_SCALE_LOOKUP:            # (2(7x, i5)): table extents
                    n_tmp, n_pre = self.t_lookup.shape
                    L.append(f"       {n_pre:5d}       {n_tmp:5d}")
                elif fnc == abi.IP_SCALE_T_LOOKUP:        # (14x, i5)
                    L.append(" " * 14 + f"{int(self.n_t_lookup_gas[g]):5d}")
                else:
                    L.append(f"      {e(self.p_ref[g, b])}      {e(self.t_ref[g, b])}")
                for kk in range(nk):
                    # read_spectrum.F90 block 5: (2(3x, 1pe16.9), i3, :, (t42, 1pe16.9, 3x, 1pe16.9))
                    vals = [self.scale[v, kk, b, g] for v in range(N_SCALE_VARIABLE.get(fnc, 0))]
                    line = f"   {e(self.k[kk, b, g])}   {e(self.w[kk, b, g])}  0"
                    if not vals:
                        L.append(line)
                    for q in range(0, len(vals), 2):
                        pair = "   ".join(e(v) for v in vals[q:q + 2])
                        L.append((line if q == 0 else " " * 41) + pair)
        L.append("*END")
        if self.thermal_coeff is not None:
            L.append("*BLOCK: TYPE =    6: SUBTYPE =    0: VERSION =    0")
            L.append("Thermal source function.")
            L.append(f"Degree of polynomial = {self.n_deg_fit:5d}: Reference temperature = {e(self.t_ref_planck)}")
            L.append("Coefficients in each band.")
            L.append("Band          w/m2")
            for b in range(self.n_band):
                L.append(f"{b + 1:5d}   " + " ".join(e(c) for c in self.thermal_coeff[:, b]))
            L.append("*END")
        if self.n_band_continuum is not None:
            L.append("*BLOCK: TYPE =    8: SUBTYPE =    0: VERSION =    0")
            L.append("Continuum absorbers in each interval")
            L.append("(The number is the indexing number of each type as set out")
            L.append(" in the file continuum.pcf.)")
            L.append("A zero indicates that there in no continuum absorption in the interval.")
            L.append("Band         Number of active continua followed by indexing numbers")
            for b in range(self.n_band):
                n = int(self.n_band_continuum[b])
                L.append(f"{b + 1:5d}       {n:5d}")
                if n:
                    L.append("     " + "".join(f"  {int(self.index_continuum[b, j]):3d}" for j in range(n)))
            L.append("Indexing numbers of gases for continua:")
            L.append(f"     Index of water = {int(self.index_water):5d}")
            L.append("*END")
            L.append("*BLOCK: TYPE =    9: SUBTYPE =    0: VERSION =    0")
            L.append("Continuum absorption coefficients: (units: m5/(kg.mol))")
            L.append("Band        Continuum   Scaling function followed by reference pressure and")
            L.append("             temperature, extinction, and scaling parameters.")
            for b in range(self.n_band):
                for j in range(int(self.n_band_continuum[b])):
                    fnc = int(self.i_scale_fnc_cont[b, j])
                    L.append(f"{b + 1:5d}       {int(self.index_continuum[b, j]):5d}       {fnc:5d}")
                    L.append(f"      {e(self.p_ref_cont[j, b])}      {e(self.t_ref_cont[j, b])}")
                    vals = [self.scale_cont[v, b, j] for v in range(N_SCALE_VARIABLE.get(fnc, 0))]
                    # (6x, 1pe16.9, (t23, 2(6x, 1pe16.9)))
                    line = f"      {e(self.k_cont[b, j])}"
                    for q in range(0, max(len(vals), 1), 2):
                        pair = "".join(f"      {e(v)}" for v in vals[q:q + 2])
                        L.append((line if q == 0 else " " * 22) + pair)
            L.append("*END")
        if self.l_doppler is not None:
            L.append("*BLOCK: TYPE =   13: SUBTYPE =    0: VERSION =    0")
            L.append("Doppler broadening coefficients for the gases")
            L.append("Species    Doppler flag   Doppler coefficient")
            for i in range(self.n_absorb):
                flag = "T" if self.l_doppler[i] else "F"
                L.append(f"{i + 1:5d}       {flag:>6s}         {self.doppler_cor[i]:12.5E}")
            L.append("*END")
        # blocks 10 and 12 in the fixed layout read_spectrum.F90 reads
        # (read_block_10_0_2: 4(4x, 1pe12.5) per line, six significant digits)
        for blk, pre, parm, ids, label in ((10, "drop", self.drop_parm_list, self.i_drop_parm, "droplets"),
                                           (12, "ice", self.ice_parm_list, self.i_ice_parm, "ice crystals")):
            if parm is None:
                continue
            npar = getattr(self, pre + "_n_parm")
            nphf = getattr(self, pre + "_n_phf")
            lo, hi = getattr(self, pre + "_parm_min_dim"), getattr(self, pre + "_parm_max_dim")
            word = "Number" if blk == 10 else "number"
            for t in range(parm.shape[2]):
                if int(ids[t]) <= 0:
                    continue
                n = int(npar[t]) if npar is not None else parm.shape[0]
                L.append(f"*BLOCK: TYPE = {blk:4d}: SUBTYPE =    0: VERSION =    2")
                L.append(f"Parametrized scattering data for {label}.")
                L.append(f" Type number of {label} = {t + 1:5d}")
                L.append(f"Index of parametrization scheme = {int(ids[t]):5d}:   {word} of parameters = {n:5d}")
                L.append(f"Number of moments of the phase function = {int(nphf[t]) if nphf is not None else 1:5d}")
                rlo = float(lo[t]) if lo is not None else 1.0e-07
                rhi = float(hi[t]) if hi is not None else 1.0e-03
                L.append(f"Range of validity of parametrization = {rlo:12.5E} -- {rhi:12.5E}")
                for b in range(self.n_band):
                    L.append(f"Band = {b + 1:5d}     Fitting parameters:")
                    vals = parm[:n, b, t]
                    for q in range(0, n, 4):
                        L.append("".join(f"    {v:12.5E}" for v in vals[q:q + 4]))
                L.append("*END")
        # block 11: dry species as subtype 0, moist ones as subtype 1, both
        # version 2 (read_block_11_0_2 / read_block_11_1_2 layouts)
        if self.aerosol_abs is not None:
            for j in range(self.aerosol_abs.shape[1]):
                nphf = int(self.n_aerosol_phf_term[j])
                nh = int(self.nhumidity[j])
                moist = int(self.i_aerosol_parm[j]) in (2, 5)
                L.append(f"*BLOCK: TYPE =   11: SUBTYPE =    {1 if moist else 0}: VERSION =    2")
                L.append(f"Scattering parameters for {'moist' if moist else 'dry'} aerosols.")
                L.append(f"Index of species = {j + 1:5d}  Aerosol")
                if moist:
                    L.append(f"Number of humidity values = {nh:3d}")
                L.append(f"Number of terms in phase function = {nphf:5d}")
                if not moist:
                    L.append("Band        Absorption          Scattering          Phase fnc")
                    L.append("            (m2.kg-1)           (m2.kg-1)")
                for b in range(self.n_band):
                    if moist:
                        L.append(f"Band = {b + 1:4d}")
                        L.append("        Humidity            Absorption         Scattering          Phase fnc.")
                        L.append("                            (m2.kg-1)          (m2.kg-1)")
                        for h in range(nh):
                            vals = [self.aerosol_humidities[h, j], self.aerosol_abs[h, j, b],
                                    self.aerosol_scat[h, j, b]] + list(self.aerosol_phf[h, :nphf, j, b])
                            L.append("".join(f"    {v:16.9E}" for v in vals))
                    else:
                        vals = [self.aerosol_abs[0, j, b], self.aerosol_scat[0, j, b]] + \
                            list(self.aerosol_phf[0, :nphf, j, b])
                        L.append(f"{b + 1:5d}" + "".join(f"    {v:16.9E}" for v in vals))
                L.append("*END")
        with open(path, "w") as fh:
            fh.write("\n".join(L) + "\n")

    def write_k_file(self, path) -> None:
        """Write the lookup tables in the '_k' companion file's record layouts,
        in the order read_spectrum.F90:1420-1560 reads them."""
        def rows(vals):
            out = []
            vals = list(vals)
            for q in range(0, len(vals), 6):
                out.append("".join(f"{v:13.6E}" for v in vals[q:q + 6]))
            return out
        L = []
        recs = [(b, int(self.index_absorb[j, b]) - 1) for b in range(self.n_band)
                for j in range(int(self.n_band_absorb[b]))]
        if self.k_lookup is not None:
            n_tmp, n_pre = self.t_lookup.shape
            L += ["*BLOCK: k-table", "", f"Lookup table: {n_pre:4d} pressures, {n_tmp:4d} temperatures."]
            for ip in range(n_pre):
                L += rows([np.exp(self.p_lookup[ip])] + list(self.t_lookup[:, ip]))
            sb = self.index_sb is not None and self.k_lookup_sb is not None
            if sb:
                L += ["", f"Gas fractions:{self.gf_lookup.size:4d}"] + rows(self.gf_lookup)
            for b, g in recs:
                if int(self.i_scale_fnc[b, g]) != abi.IP_SCALE_LOOKUP:
                    continue
                nk = int(self.i_band_k[b, g])
                L += ["", f"Band: {b + 1:4d}, gas: {g + 1:4d}, k-terms: {nk:4d}"]
                for t in range(nk):
                    if sb and self.index_sb[g] > 0:
                        for ig in range(self.gf_lookup.size):
                            for ip in range(n_pre):
                                L += rows(self.k_lookup_sb[:, ip, ig, t, self.index_sb[g] - 1, b])
                    else:
                        for ip in range(n_pre):
                            L += rows(self.k_lookup[:, ip, t, g, b])
            L.append("*END")
        if self.k_t_lookup_gas is not None:
            ndt = self.t_lookup_gas.shape[0]
            L += ["*BLOCK: temperature k-tables", "", f"nd_t =   {ndt:4d}"]
            for g in range(self.n_absorb):
                if int(self.n_t_lookup_gas[g]) > 1:
                    n = int(self.n_t_lookup_gas[g])
                    L += ["", "Temperatures of absorber   " + f"{n:4d}"] + rows(self.t_lookup_gas[:n, g])
            for b, g in recs:
                if int(self.i_scale_fnc[b, g]) != abi.IP_SCALE_T_LOOKUP:
                    continue
                n = int(self.n_t_lookup_gas[g])
                L += ["", f"Band: {b + 1:4d}, gas: {g + 1:4d}"]
                for t in range(int(self.i_band_k[b, g])):
                    L += rows(self.k_t_lookup_gas[:n, t, g, b])
            L.append("*END")
        Path(path).write_text("\n".join(L) + "\n")

    def write_wenyi_data(self, path) -> None:
        """Write the Wen-Yi tables as their data file (the form
        read_wenyi_tables and socgpu_spectrum_load_ext read)."""
        from socrates_gb300 import wenyi
        wenyi.write_data(path, {k: getattr(self, k) for k in ("wenyi_plg", "wenyi_ttb", "wenyi_tto",
                                                                "wenyi_gk250b", "wenyi_gk4", "wenyi_gk6")})

    @classmethod
    def read_text(cls, path, name: str | None = None, k_path=None) -> "Spectrum":
        """Read a spectral file in the reference's text format: blocks 0
        (summary, versions 1 and 2), 1 (band limits), 2 (solar spectrum), 3
        (Rayleigh), 4 (absorbers per band), 5 (k-terms), 6 (Planck
        polynomial), 8 and 9 (continua), 13 (Doppler broadening) and the
        Pade droplet/ice blocks 10 and 12 (parametrisations 5 and 20); record
        layouts of read_spectrum.F90 (blocks 0-13).  Other blocks (surface
        properties, aerosols, other cloud parametrisations) are skipped.
        The lookup tables of block 5 come from the '_k' companion file (path +
        '_k' unless k_path is given)."""
        text = open(path).read().splitlines()
        blocks = []
        cur = None
        for ln in text:
            if ln.startswith("*BLOCK"):
                parts = ln.replace(":", " ").replace("=", " ").split()
                cur = {"type": int(parts[2]), "subtype": int(parts[4]), "version": int(parts[6]), "lines": []}
                blocks.append(cur)
            elif ln.startswith("*END"):
                cur = None
            elif cur is not None:
                cur["lines"].append(ln)
        by = {}
        for bl in blocks:
            by.setdefault(bl["type"], []).append(bl)

        def after_eq(line):
            return line.split("=")[1].split()[0]

        # block 0: summary
        b0 = by[0][0]["lines"]
        n_band = n_abs = None
        types = []
        for q, ln in enumerate(b0):
            u = ln.upper()
            if "SPECTRAL BANDS" in u:
                n_band = int(after_eq(ln))
            elif "GASEOUS ABSORBERS" in u:
                n_abs = int(after_eq(ln))
            elif "INDEXING NUMBERS AND ABSORBERS" in u or ("INDEXING NUMBERS" in u and "ABSORBER" in u
                                                            and "AEROSOL" not in u):
                for r in b0[q + 2:q + 2 + n_abs]:
                    types.append(int(r.split()[1]))
        # block 1: band limits
        wl = np.zeros((n_band, 2))
        for r in by[1][0]["lines"][3:3 + n_band]:
            v = r.split()
            wl[int(v[0]) - 1] = float(v[1]), float(v[2])

        def band_values(blk, skip):
            if blk not in by:
                return None
            out = np.zeros(n_band)
            for r in by[blk][0]["lines"][skip:]:
                v = r.split()
                if len(v) >= 2 and v[0].isdigit():
                    out[int(v[0]) - 1] = float(v[1])
            return out
        sol = band_values(2, 2)
        ray = band_values(3, 3)
        # block 4: absorbers in each band (token stream after 5 header lines);
        # version 1 adds each band's overlap method (read_spectrum.F90 block 4_0_1)
        toks = " ".join(by[4][0]["lines"][5:]).split()
        with_overlap = by[4][0]["version"] >= 1
        nba = np.zeros(n_band, np.int32)
        i_ovl = np.zeros(n_band, np.int32) if with_overlap else None
        ia = np.zeros((max(1, n_abs), n_band), np.int32)
        q = 0
        for _ in range(n_band):
            b = int(toks[q]) - 1
            nba[b] = int(toks[q + 1])
            q += 2
            if with_overlap:
                i_ovl[b] = int(toks[q])
                q += 1
            for j in range(nba[b]):
                ia[j, b] = int(toks[q])
                q += 1
        # block 5: k-terms, fixed columns (2(3x, 1pe16.9), i3, :, (t42, 1pe16.9, 3x, 1pe16.9)).
        # Version 1 may first list the self-broadened absorbers
        # (read_spectrum.F90:1268-1300); lookup-table records give the table
        # extents in place of the reference pressure and temperature.
        b5 = by[5][0]["lines"]
        isb = None
        q0 = 4
        for q, ln in enumerate(b5):
            if ln.strip().startswith("Self-broadened indexing numbers"):
                vals, r = [], q + 2
                while len(vals) < n_abs:
                    vals += [int(x) for x in b5[r].split()]
                    r += 1
                isb = np.array(vals[:n_abs], np.int32)
            if ln.startswith("Band        Gas, Number of k-terms"):
                q0 = q + 3
                break
        recs = []
        lines = b5[q0:]
        q = 0
        nd_k, nsv_max = 1, 4
        n_pre = n_tmp = 0
        while q < len(lines):
            parts = lines[q].split()
            if len(parts) < 5:
                q += 1
                continue
            b, g, nk, sk, fnc = (int(x) for x in parts[:5])
            p_ref = t_ref = 0.0
            if fnc == abi.IP_SCALE_LOOKUP:
                n_pre, n_tmp = (int(x) for x in lines[q + 1].split()[:2])
            elif fnc != abi.IP_SCALE_T_LOOKUP:
                p_ref, t_ref = (float(x) for x in lines[q + 1].split()[:2])
            q += 2
            nsv = N_SCALE_VARIABLE.get(fnc, 0)
            terms = []
            for _ in range(nk):
                ln = lines[q]
                k_ = float(ln[3:19])
                w_ = float(ln[22:38])
                vals = []
                col = ln
                while len(vals) < nsv:
                    for a, z in ((41, 57), (60, 76)):
                        if len(vals) < nsv and len(col) > a and col[a:z].strip():
                            vals.append(float(col[a:z]))
                    if len(vals) < nsv:
                        q += 1
                        col = lines[q]
                q += 1
                terms.append((k_, w_, vals))
            recs.append((b - 1, g - 1, nk, sk, fnc, p_ref, t_ref, terms))
            nd_k = max(nd_k, nk)
            nsv_max = max(nsv_max, nsv)
        tables = {}
        if any(r[4] in (abi.IP_SCALE_LOOKUP, abi.IP_SCALE_T_LOOKUP) for r in recs):
            kp = Path(k_path) if k_path is not None else Path(str(path) + "_k")
            if not kp.exists():
                raise ValueError(f"the k-term lookup tables of block 5 are in {kp}, which cannot be read")
            tables = _read_k_file(kp, n_band, n_abs, nd_k, recs, ia, nba, isb, n_pre, n_tmp)
        ibk = np.zeros((n_band, n_abs), np.int32)
        isk = np.zeros((n_band, n_abs), np.int32)
        isf = np.zeros((n_band, n_abs), np.int32)
        kk = np.zeros((nd_k, n_band, n_abs))
        ww = np.zeros((nd_k, n_band, n_abs))
        sc = np.zeros((nsv_max, nd_k, n_band, n_abs))
        pr = np.zeros((n_abs, n_band))
        tr = np.zeros((n_abs, n_band))
        for b, g, nk, sk, fnc, p_ref, t_ref, terms in recs:
            ibk[b, g], isk[b, g], isf[b, g] = nk, sk, fnc
            pr[g, b], tr[g, b] = p_ref, t_ref
            for t, (k_, w_, vals) in enumerate(terms):
                kk[t, b, g], ww[t, b, g] = k_, w_
                sc[:len(vals), t, b, g] = vals
        # block 6: Planck polynomial
        tc, ndeg, tref = None, 0, 0.0
        if 6 in by:
            b6 = by[6][0]["lines"]
            hdr = next(ln for ln in b6 if "=" in ln)
            ndeg = int(hdr.split("=")[1].split(":")[0])
            tref = float(hdr.split("=")[2])
            vals = " ".join(b6[b6.index(hdr) + 3:]).split()
            tc = np.zeros((ndeg + 1, n_band))
            q = 0
            for _ in range(n_band):
                b = int(vals[q]) - 1
                tc[:, b] = [float(x) for x in vals[q + 1:q + 2 + ndeg]]
                q += ndeg + 2
        # blocks 8 and 9: continua
        cont = {}
        if 8 in by:
            b8 = by[8][0]["lines"]
            toks = []
            iw = 0
            for ln in b8[5:]:
                if "=" in ln:
                    iw = int(after_eq(ln))
                elif ln.strip() and ln.strip()[0].isdigit():
                    toks += ln.split()
            nbc = np.zeros(n_band, np.int32)
            idx = {}
            q = 0
            while q < len(toks):
                b = int(toks[q]) - 1
                n = int(toks[q + 1])
                nbc[b] = n
                idx[b] = [int(x) for x in toks[q + 2:q + 2 + n]]
                q += 2 + n
            ndc = max(1, int(nbc.max()))
            ic = np.zeros((n_band, ndc), np.int32)
            for b, v in idx.items():
                ic[b, :len(v)] = v
            fc = np.zeros((n_band, ndc), np.int32)
            kc = np.zeros((n_band, ndc))
            scc = np.zeros((max(nsv_max, 3), n_band, ndc))
            prc = np.zeros((ndc, n_band))
            trc = np.zeros((ndc, n_band))
            if 9 in by:
                toks = " ".join(by[9][0]["lines"][3:]).split()
                q = 0
                while q < len(toks):
                    b, ci, fnc = int(toks[q]) - 1, int(toks[q + 1]), int(toks[q + 2])
                    j = list(ic[b]).index(ci)
                    fc[b, j] = fnc
                    prc[j, b], trc[j, b] = float(toks[q + 3]), float(toks[q + 4])
                    kc[b, j] = float(toks[q + 5])
                    nsv = N_SCALE_VARIABLE.get(fnc, 0)
                    scc[:nsv, b, j] = [float(x) for x in toks[q + 6:q + 6 + nsv]]
                    q += 6 + nsv
            cont = dict(n_band_continuum=nbc, index_continuum=_f(ic, np.int32), index_water=iw,
                        i_scale_fnc_cont=_f(fc, np.int32), k_cont=_f(kc, np.float64),
                        scale_cont=_f(scc, np.float64), p_ref_cont=_f(prc, np.float64),
                        t_ref_cont=_f(trc, np.float64))
        # block 13: Doppler broadening
        ldop = dcor = None
        if 13 in by:
            ldop = np.zeros(n_abs, np.int32)
            dcor = np.zeros(n_abs)
            for ln in by[13][0]["lines"][2:]:
                v = ln.split()
                if len(v) >= 3 and v[0].isdigit():
                    i = int(v[0]) - 1
                    ldop[i] = 1 if v[1].upper().startswith("T") else 0
                    dcor[i] = float(v[2])

        def cloud_sets(blk):
            """Blocks 10 or 12 (read_block_10_0_2 / read_block_12_0_2 of
            read_spectrum.F90): every set at its type number, with its scheme,
            phase-function moments and range of validity."""
            found = {}
            for bl in by.get(blk, []):
                lines = bl["lines"]
                head = next((ln for ln in lines if "=" in ln and "PARAMETERS" in ln.upper()), None)
                tline = next((ln for ln in lines if "TYPE NUMBER" in ln.upper()), None)
                if head is None or tline is None:
                    continue
                ty = int(tline.split("=")[1].split()[0])
                scheme = int(head.split("=")[1].split(":")[0])
                npar = int(head.split("=")[2])
                nphf, lo, hi = 1, 0.0, 0.0
                vals = []
                for ln in lines[lines.index(head) + 1:]:
                    u = ln.upper()
                    if "MOMENTS" in u:
                        nphf = int(ln.split("=")[1].split()[0])
                        continue
                    if "RANGE" in u:
                        r = ln.split("=")[1].split("--")
                        lo, hi = float(r[0]), float(r[1])
                        continue
                    if not any(ch.isdigit() for ch in ln):
                        continue
                    if "BAND" in u and "=" in ln:
                        vals.append(ln.split("=")[1].split()[0])
                    else:
                        vals += ln.split()
                arr = np.zeros((npar, n_band))
                q = 0
                for _ in range(n_band):
                    b = int(vals[q]) - 1
                    arr[:, b] = [float(x) for x in vals[q + 1:q + 1 + npar]]
                    q += npar + 1
                found[ty] = (scheme, npar, nphf, lo, hi, arr)
            if not found:
                return None
            nt = max(found)
            ncp = max(v[1] for v in found.values())
            parm = np.zeros((ncp, n_band, nt))
            ids, npars, nphfs = (np.zeros(nt, np.int32) for _ in range(3))
            lo, hi = np.zeros(nt), np.zeros(nt)
            for ty, (scheme, npar, nphf, a, b, arr) in found.items():
                parm[:npar, :, ty - 1] = arr
                ids[ty - 1], npars[ty - 1], nphfs[ty - 1] = scheme, npar, nphf
                lo[ty - 1], hi[ty - 1] = a, b
            return np.asfortranarray(parm), ids, npars, nphfs, lo, hi

        # block 11: classic aerosol species; block 0 gives their number and
        # type numbers (read_spectrum.F90:2335-2640)
        aerosol = {}
        n_aer, aer_types = 0, []
        for q, ln in enumerate(b0):
            u = ln.upper()
            if "NUMBER OF AEROSOLS" in u:
                n_aer = int(after_eq(ln))
            elif "INDEXING NUMBERS OF AEROSOLS" in u:
                for r in b0[q + 2:q + 2 + n_aer]:
                    aer_types.append(int(r.split()[1]))
        if n_aer > 0 and 11 in by:
            def numeric(line):
                try:
                    return [float(x.replace("D", "E").replace("d", "e")) for x in line.split()]
                except ValueError:
                    return None
            parsed = {}
            for bl in by[11]:
                lines = bl["lines"]
                sp_i = nh = None
                nphf = 1
                for ln in lines:
                    u = ln.upper()
                    if "INDEX OF SPECIES" in u:
                        sp_i = int(after_eq(ln))
                    elif "NUMBER OF HUMIDITY" in u:
                        nh = int(after_eq(ln))
                    elif "NUMBER OF TERMS IN PHASE FUNCTION" in u:
                        nphf = int(after_eq(ln))
                toks = []
                for ln in lines:
                    v = numeric(ln)
                    if v:
                        toks += v
                moist = bl["subtype"] == 1
                rows = nh if moist else 1
                per = (3 + nphf) * rows
                if len(toks) < per * n_band:
                    raise ValueError(f"{path}: aerosol species {sp_i}: short of values")
                parsed[sp_i] = (moist, rows, nphf, np.array(toks[:per * n_band]).reshape(n_band, rows, 3 + nphf))
            ndh = max(v[1] for v in parsed.values())
            ndp = max(v[2] for v in parsed.values())
            hum = np.zeros((ndh, n_aer))
            ab, scat = np.zeros((ndh, n_aer, n_band)), np.zeros((ndh, n_aer, n_band))
            phf = np.zeros((ndh, ndp, n_aer, n_band))
            parm, nhum, nterm = (np.zeros(n_aer, np.int32) for _ in range(3))
            for sp_i, (moist, rows, nphf, arr) in parsed.items():
                j = sp_i - 1
                nterm[j] = nphf
                nhum[j] = rows if moist else 0
                parm[j] = (2 if nphf == 1 else 5) if moist else (1 if nphf == 1 else 4)
                for b in range(n_band):
                    if moist:
                        hum[:rows, j] = arr[b, :, 0]
                    ab[:rows, j, b] = arr[b, :, 1]
                    scat[:rows, j, b] = arr[b, :, 2]
                    phf[:rows, :nphf, j, b] = arr[b, :, 3:3 + nphf]
            aerosol = dict(type_aerosol=np.array(aer_types, np.int32), i_aerosol_parm=parm, nhumidity=nhum,
                           n_aerosol_phf_term=nterm, aerosol_humidities=_f(hum, np.float64),
                           aerosol_abs=_f(ab, np.float64), aerosol_scat=_f(scat, np.float64),
                           aerosol_phf=_f(phf, np.float64))

        cloud = {}
        for blk, pre in ((10, "drop"), (12, "ice")):
            r = cloud_sets(blk)
            if r is not None:
                parm, ids, npars, nphfs, lo, hi = r
                cloud.update({f"{pre}_parm_list": parm, f"i_{pre}_parm": ids, f"{pre}_n_parm": npars,
                              f"{pre}_n_phf": nphfs, f"{pre}_parm_min_dim": lo, f"{pre}_parm_max_dim": hi})
        return cls(n_band=n_band, wavelength_short=wl[:, 0], wavelength_long=wl[:, 1],
                   type_absorb=np.array(types, np.int32), n_band_absorb=nba, index_absorb=ia,
                   i_band_k=ibk, i_scale_k=isk, i_scale_fnc=isf, k=_f(kk, np.float64), w=_f(ww, np.float64),
                   scale=_f(sc, np.float64), p_ref=pr, t_ref=tr, solar_flux_band=sol, rayleigh_coeff=ray,
                   n_deg_fit=ndeg, t_ref_planck=tref, thermal_coeff=tc,
                   l_doppler=ldop, doppler_cor=dcor, name=name or str(path),
                   i_overlap=i_ovl, **cont, **tables, **cloud, **aerosol)
