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

import numpy as np

from . import abi

GAS_NAMES = {1: "Water Vapour", 2: "Carbon Dioxide", 3: "Ozone", 4: "Dinitrogen Oxide", 5: "Carbon monoxide",
             6: "Methane", 7: "Oxygen"}


def _f(a, dtype):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


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
    drop_parm_list: np.ndarray | None = None # (16, n_band, n_drop_type)
    i_drop_parm: np.ndarray | None = None    # (n_drop_type)
    ice_parm_list: np.ndarray | None = None  # (16, n_band, n_ice_type)
    i_ice_parm: np.ndarray | None = None
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
        d.l_doppler = None
        d.doppler_cor = None
        if self.thermal_coeff is not None:
            d.n_deg_fit = self.n_deg_fit
            d.t_ref_planck = self.t_ref_planck
            d.nd_thermal_coeff = self.thermal_coeff.shape[0]
            d.thermal_coeff = dp(self.thermal_coeff)
        if self.drop_parm_list is not None:
            d.nd_cloud_parameter = self.drop_parm_list.shape[0]
            d.nd_drop_type = self.drop_parm_list.shape[2]
            d.drop_parm_list = dp(self.drop_parm_list)
            d.i_drop_parm = ip(self.i_drop_parm)
            d.l_drop_type = ip(np.ones(d.nd_drop_type, np.int32))
        if self.ice_parm_list is not None:
            d.nd_cloud_parameter = max(d.nd_cloud_parameter, self.ice_parm_list.shape[0])
            d.nd_ice_type = self.ice_parm_list.shape[2]
            d.ice_parm_list = dp(self.ice_parm_list)
            d.i_ice_parm = ip(self.i_ice_parm)
            d.l_ice_type = ip(np.ones(d.nd_ice_type, np.int32))
        self._keep = keep
        return d

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
        L.append(f"Total number of aerosols = {0:5d}")
        L.append("List of indexing numbers and absorbers.")
        L.append("Index       Absorber(identifier and name)")
        for i, t in enumerate(self.type_absorb):
            L.append(f"{i + 1:5d}       {int(t):5d}       {GAS_NAMES.get(int(t), 'Gas'):20s}")
        L.append("List of indexing numbers of aerosols.")
        L.append("Index       Aerosol(type number and name)")
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
            L.append("Rayleigh mass scattering coefficients.")
            L.append("Band        Rayleigh coefficient (m2/kg)")
            for b in range(self.n_band):
                L.append(f"{b + 1:5d}       {e(self.rayleigh_coeff[b])}")
            L.append("*END")
        L.append("*BLOCK: TYPE =    4: SUBTYPE =    0: VERSION =    0")
        L.append("Gaseous absorbers in each interval")
        L.append("(The number is the indexing number of the species as set out")
        L.append(" in the summary block 0.)")
        L.append("A zero indicates that there in no gaseous absorption in the interval.")
        L.append("Band        Number of active absorbers followed by indexing numbers")
        for b in range(self.n_band):
            L.append(f"{b + 1:5d}       {int(self.n_band_absorb[b]):5d}")
            if self.n_band_absorb[b] > 0:
                L.append("   " + "".join(f"{int(self.index_absorb[j, b]):5d}" for j in range(int(self.n_band_absorb[b]))))
        L.append("*END")
        L.append("*BLOCK: TYPE =    5: SUBTYPE =    0: VERSION =    0")
        L.append("Exponential sum fiting coefficients: (exponents: m2/kg)")
        L.append("Band        Gas, Number of k-terms, Scaling type and scaling function,")
        L.append("             followed by reference pressure and temperature,")
        L.append("                   k-terms, weights and scaling parameters.")
        nsv = {0: 0, 1: 2, 2: 3, 3: 4}
        for b in range(self.n_band):
            for j in range(int(self.n_band_absorb[b])):
                g = int(self.index_absorb[j, b]) - 1
                nk = int(self.i_band_k[b, g])
                fnc = int(self.i_scale_fnc[b, g])
                L.append(f"{b + 1:5d}       {g + 1:5d}       {nk:5d}       {int(self.i_scale_k[b, g]):5d}       {fnc:5d}")
                L.append(f"      {e(self.p_ref[g, b])}      {e(self.t_ref[g, b])}")
                for kk in range(nk):
                    sc = "".join(f"   {e(self.scale[v, kk, b, g])}" for v in range(nsv.get(fnc, 0)))
                    L.append(f"   {e(self.k[kk, b, g])}   {e(self.w[kk, b, g])}  1{sc}")
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
        for blk, parm, ids, label in ((10, self.drop_parm_list, self.i_drop_parm, "droplets"),
                                      (12, self.ice_parm_list, self.i_ice_parm, "ice crystals")):
            if parm is None:
                continue
            for t in range(parm.shape[2]):
                L.append(f"*BLOCK: TYPE = {blk:4d}: SUBTYPE =    0: VERSION =    2")
                L.append(f"Parametrized scattering data for {label}.")
                L.append(f" Type number = {t + 1:5d}")
                L.append(f"Index of parametrization scheme = {int(ids[t]):5d}:   Number of parameters = {parm.shape[0]:5d}")
                L.append("Band        Parameters")
                for b in range(self.n_band):
                    L.append(f"{b + 1:5d}   " + " ".join(e(c) for c in parm[:, b, t]))
                L.append("*END")
        with open(path, "w") as fh:
            fh.write("\n".join(L) + "\n")

    @classmethod
    def read_text(cls, path, name: str | None = None) -> "Spectrum":
        """Read blocks 0-6, 10 and 12 of a spectral file in the text format.

        Only what write_text produces is guaranteed; lookup-table k scaling
        (ip_scale_lookup, '_k' files) and continua are not read."""
        text = open(path).read().splitlines()
        blocks = []
        cur = None
        for ln in text:
            if ln.startswith("*BLOCK"):
                parts = ln.replace(":", " ").replace("=", " ").split()
                cur = {"type": int(parts[2]), "lines": []}
                blocks.append(cur)
            elif ln.startswith("*END"):
                cur = None
            elif cur is not None:
                cur["lines"].append(ln)
        by = {}
        for bl in blocks:
            by.setdefault(bl["type"], []).append(bl["lines"])
        b0 = by[0][0]
        n_band = int(b0[1].split("=")[1])
        n_abs = int(b0[2].split("=")[1])
        nd_k = int(b0[3].split("=")[1])
        types = [int(l.split()[1]) for l in b0[7:7 + n_abs]]
        wl = np.array([[float(x) for x in l.split()[1:3]] for l in by[1][0][3:3 + n_band]])
        sol = None
        if 2 in by:
            sol = np.array([float(l.split()[1]) for l in by[2][0][2:2 + n_band]])
        ray = None
        if 3 in by:
            ray = np.array([float(l.split()[1]) for l in by[3][0][2:2 + n_band]])
        # block 4
        toks = " ".join(by[4][0][5:]).split()
        nba = np.zeros(n_band, np.int32)
        ia = np.zeros((max(1, n_abs), n_band), np.int32)
        q = 0
        for b in range(n_band):
            q += 1  # band index
            nba[b] = int(toks[q]); q += 1
            for j in range(nba[b]):
                ia[j, b] = int(toks[q]); q += 1
        # block 5
        ibk = np.zeros((n_band, n_abs), np.int32)
        isk = np.zeros((n_band, n_abs), np.int32)
        isf = np.zeros((n_band, n_abs), np.int32)
        kk = np.zeros((nd_k, n_band, n_abs))
        ww = np.zeros((nd_k, n_band, n_abs))
        sc = np.zeros((4, nd_k, n_band, n_abs))
        pr = np.zeros((n_abs, n_band))
        tr = np.zeros((n_abs, n_band))
        lines = by[5][0][4:]
        q = 0
        nsv = {0: 0, 1: 2, 2: 3, 3: 4}
        while q < len(lines):
            parts = lines[q].split()
            if not parts:
                q += 1
                continue
            b, g, nk, sk, fnc = (int(x) for x in parts[:5])
            b -= 1
            g -= 1
            ibk[b, g], isk[b, g], isf[b, g] = nk, sk, fnc
            pr[g, b], tr[g, b] = (float(x) for x in lines[q + 1].split()[:2])
            for t in range(nk):
                v = lines[q + 2 + t].split()
                kk[t, b, g], ww[t, b, g] = float(v[0]), float(v[1])
                for s in range(nsv.get(fnc, 0)):
                    sc[s, t, b, g] = float(v[3 + s])
            q += 2 + nk
        tc = None
        ndeg = 0
        tref = 0.0
        if 6 in by:
            hdr = by[6][0][1]
            ndeg = int(hdr.split(":")[0].split("=")[1])
            tref = float(hdr.split(":")[1].split("=")[1])
            tc = np.zeros((ndeg + 1, n_band))
            vals = " ".join(by[6][0][4:]).split()
            q = 0
            for b in range(n_band):
                q += 1
                tc[:, b] = [float(x) for x in vals[q:q + ndeg + 1]]
                q += ndeg + 1

        def cloud(blk):
            if blk not in by:
                return None, None
            sets, ids = [], []
            for lines in by[blk]:
                ids.append(int(lines[2].split("=")[1].split(":")[0]))
                npar = int(lines[2].split("=")[2])
                arr = np.zeros((npar, n_band))
                vals = " ".join(lines[4:]).split()
                q = 0
                for b in range(n_band):
                    q += 1
                    arr[:, b] = [float(x) for x in vals[q:q + npar]]
                    q += npar
                sets.append(arr)
            return np.asfortranarray(np.stack(sets, axis=2)), np.array(ids, np.int32)

        dpl, dids = cloud(10)
        ipl, iids = cloud(12)
        return cls(n_band=n_band, wavelength_short=wl[:, 0], wavelength_long=wl[:, 1],
                   type_absorb=np.array(types, np.int32), n_band_absorb=nba, index_absorb=ia,
                   i_band_k=ibk, i_scale_k=isk, i_scale_fnc=isf, k=_f(kk, np.float64), w=_f(ww, np.float64),
                   scale=_f(sc, np.float64), p_ref=pr, t_ref=tr, solar_flux_band=sol, rayleigh_coeff=ray,
                   n_deg_fit=ndeg, t_ref_planck=tref, thermal_coeff=tc, drop_parm_list=dpl, i_drop_parm=dids,
                   ice_parm_list=ipl, i_ice_parm=iids, name=name or str(path))
