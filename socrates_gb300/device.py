"""Device-resident inputs for socgpu_radiance_calc_device.

PyTorch is plumbing here: it allocates HBM, owns the streams and records
CUDA events.  Arrays keep the reference's Fortran layout (flattened in
column-major order), so the same leading extents apply as on the host.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .radiance import Control, Marshal, McicaState, RadianceError, load_library, register_spectrum
from .spectrum import Spectrum


def _to_dev(a, dtype=None):
    import torch
    if a is None:
        return None
    arr = np.asfortranarray(a if dtype is None else np.asarray(a, dtype=dtype))
    flat = arr.ravel(order="F")
    return torch.from_numpy(np.ascontiguousarray(flat)).to("cuda", non_blocking=False)


class DeviceCase:
    """One radiance_calc problem with every array resident on the GPU."""

    def __init__(self, control: Control, spectrum: Spectrum, col, mcica: McicaState | None = None,
                 id_cloud_top: int = 1, keep_host: bool = True):
        import torch
        self.lib = load_library()
        self.handle = register_spectrum(spectrum)
        self.host = Marshal(control, spectrum, col, mcica, id_cloud_top)
        m = self.host
        self.tensors = {}
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)

        def dev(name, a, dtype=None, ctype=dp):
            if a is None:
                return None
            t = _to_dev(a, dtype)
            self.tensors[name] = t
            return C.cast(C.c_void_p(t.data_ptr()), ctype)

        self.atm = abi.Atm()
        self.atm.n_profile, self.atm.n_layer = col.n_profile, col.n_layer
        self.atm.p = dev("p", col.p)
        self.atm.t = dev("t", col.t)
        self.atm.t_level = dev("t_level", col.t_level)
        self.atm.mass = dev("mass", col.mass)
        self.atm.gas_mix_ratio = dev("gas", col.gas_mix_ratio)
        self.atm.density = dev("density", getattr(col, "density", None))
        self.bound = abi.Bound()
        self.bound.zen_0 = dev("zen_0", col.zen_0)
        self.bound.solar_irrad = dev("solar_irrad", col.solar_irrad)
        self.bound.rho_alb = dev("rho_alb", col.rho_alb)
        self.bound.t_ground = dev("t_ground", col.t_ground)
        self.aer = abi.Aer()
        if control.l_aerosol_mode and col.aer:
            self.aer.n_mode = col.aer["n_mode"]
            self.aer.mode_mix_ratio = dev("amr", col.aer["mode_mix_ratio"])
            self.aer.mode_absorption = dev("aab", col.aer["mode_absorption"])
            self.aer.mode_scattering = dev("asc", col.aer["mode_scattering"])
            self.aer.mode_asymmetry = dev("aas", col.aer["mode_asymmetry"])
        self.cld = abi.Cld()
        if mcica is not None:
            hc = m.cld
            self.cld.n_condensed, self.cld.n_cloud_type = hc.n_condensed, hc.n_cloud_type
            self.cld.type_condensed, self.cld.i_cloud_type = hc.type_condensed, hc.i_cloud_type
            self.cld.i_condensed_param, self.cld.i_condensed_type = hc.i_condensed_param, hc.i_condensed_type
            ict = id_cloud_top - 1
            cd = col.cld
            self.cld.condensed_mix_ratio = dev("cmr", cd["condensed_mix_ratio"][:, ict:, :])
            self.cld.condensed_dim_char = dev("cdc", cd["condensed_dim_char"][:, ict:, :])
            self.cld.w_cloud = dev("wc", cd["w_cloud"][:, ict:])
            self.cld.frac_cloud = dev("fc", cd["frac_cloud"][:, ict:, :])
            self.cld.n_subcol_gen, self.cld.n_subcol_req = mcica.n_subcol_gen, mcica.n_subcol_req
            self.cld.c_sub = dev("csub", mcica.c_sub)
            self.cld.frac_cloudy = dev("fcl", mcica.frac_cloudy)
            self.cld.n_subcol_cld = dev("nsc", mcica.n_subcol_cld, np.int32, ip)
            self.cld.subcol_k = dev("sk", mcica.subcol_k, np.int32, ip)
            self.cld.first_subcol_k = dev("fsk", mcica.first_subcol_k, np.int32, ip)
            self.cld.subcol_reorder = dev("sro", mcica.subcol_reorder, np.int32, ip)
        n, L = col.n_profile, col.n_layer
        z = lambda k, cnt: self.tensors.setdefault(k, torch.zeros(cnt, dtype=torch.float64, device="cuda"))
        self.radout = abi.Radout()
        for name, cnt in (("flux_up", n * (L + 1)), ("flux_down", n * (L + 1)), ("flux_direct", n * (L + 1)),
                          ("flux_div", n * L), ("heating_rate", n * L)):
            if name == "flux_direct" and control.isolir != abi.IP_SOLAR:
                continue
            if name == "flux_div" and not control.l_flux_div:
                continue
            t = z("out_" + name, cnt)
            setattr(self.radout, name, C.cast(C.c_void_p(t.data_ptr()), dp))
        self.control = m.control
        self.dimen = m.dimen
        self.n, self.L = n, L
        self.input_bytes = sum(t.numel() * t.element_size() for k, t in self.tensors.items() if not k.startswith("out_"))
        self.output_bytes = sum(t.numel() * t.element_size() for k, t in self.tensors.items() if k.startswith("out_"))
        if not keep_host:
            # the host copies are on the device now; keep only the small
            # option arrays the cloud struct points at
            m.keep = [a for a in m.keep if getattr(a, "nbytes", 0) <= 4096]
            m.flux_up = m.flux_down = m.flux_direct = m.flux_div = m.heating_rate = None

    def clone(self, precision: int) -> "DeviceCase":
        """The same problem at another precision: inputs shared, outputs new."""
        import copy
        import torch
        c = copy.copy(self)
        c.tensors = {k: v for k, v in self.tensors.items() if not k.startswith("out_")}
        c.control = type(self.control).from_buffer_copy(self.control)
        c.control.precision = precision
        c.radout = abi.Radout()
        dp = C.POINTER(C.c_double)
        for k, t in self.tensors.items():
            if k.startswith("out_"):
                nt = torch.zeros_like(t)
                c.tensors[k] = nt
                setattr(c.radout, k[4:], C.cast(C.c_void_p(nt.data_ptr()), dp))
        return c

    def tensor_bytes(self, name: str) -> int:
        t = self.tensors.get(name)
        return 0 if t is None else t.numel() * t.element_size()

    def run(self, stream_ptr: int = 0) -> None:
        msg = C.create_string_buffer(512)
        st = self.lib.socgpu_radiance_calc_device(
            C.byref(self.control), C.byref(self.dimen), self.handle, C.byref(self.atm), C.byref(self.cld),
            C.byref(self.aer), C.byref(self.bound), C.byref(self.radout), C.c_void_p(stream_ptr), msg, 512)
        if st != abi.I_NORMAL:
            raise RadianceError(st, msg.value.decode())

    def output(self, name: str) -> np.ndarray:
        t = self.tensors["out_" + name].cpu().numpy()
        rows = self.L + 1 if name in ("flux_up", "flux_down", "flux_direct") else self.L
        return t.reshape((self.n, rows), order="F")
