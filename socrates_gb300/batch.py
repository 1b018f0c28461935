"""Many radiance_calc problems replayed as one CUDA graph (socgpu_batch_*).

Each problem is a DeviceCase (device-resident arrays).  The library groups
them into kernel classes -- precision, mode (infra-red without scattering,
full scattering, McICA) and tile -- runs each class as one persistent launch
over all its columns, and captures the launches in one graph.  `tune` times
the built tiles on the batch's own data and keeps the fastest per
(precision, mode, layer count).
"""
from __future__ import annotations

import ctypes as C

from . import abi
from .device import DeviceCase
from .radiance import RadianceError, load_library


class Batch:
    def __init__(self, cases: list[DeviceCase]):
        self.lib = load_library()
        self.cases = list(cases)
        items = (abi.BatchItem * len(self.cases))()
        for it, c in zip(items, self.cases):
            it.control = C.pointer(c.control)
            it.dimen = C.pointer(c.dimen)
            it.spectrum = c.handle
            it.atm = C.pointer(c.atm)
            it.cld = C.pointer(c.cld)
            it.aer = C.pointer(c.aer)
            it.bound = C.pointer(c.bound)
            it.radout = C.pointer(c.radout)
        self.handle = C.c_void_p()
        msg = C.create_string_buffer(512)
        st = self.lib.socgpu_batch_create(items, len(self.cases), C.byref(self.handle), msg, 512)
        if st != abi.I_NORMAL:
            raise RadianceError(st, msg.value.decode())

    def run(self, stream_ptr: int = 0) -> None:
        msg = C.create_string_buffer(512)
        st = self.lib.socgpu_batch_run(self.handle, C.c_void_p(stream_ptr), msg, 512)
        if st != abi.I_NORMAL:
            raise RadianceError(st, msg.value.decode())

    def tune(self, stream_ptr: int = 0, reps: int = 3) -> None:
        msg = C.create_string_buffer(512)
        st = self.lib.socgpu_batch_tune(self.handle, C.c_void_p(stream_ptr), reps, msg, 512)
        if st != abi.I_NORMAL:
            raise RadianceError(st, msg.value.decode())

    def info(self) -> dict:
        g, n, cg = C.c_int(), C.c_longlong(), C.c_longlong()
        self.lib.socgpu_batch_info(self.handle, C.byref(g), C.byref(n), C.byref(cg))
        return {"kernel_classes": g.value, "columns": n.value, "column_gpoints": cg.value}

    def close(self) -> None:
        if self.handle:
            self.lib.socgpu_batch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tuned_tile(precision: int, mode: int, n_layer: int):
    """The tile table's entry (lanes per solve, layers per lane, warps) or None."""
    lib = load_library()
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    st = lib.socgpu_tune_get(precision, mode, n_layer, C.byref(a), C.byref(b), C.byref(c))
    return (a.value, b.value, c.value) if st == abi.I_NORMAL else None


def set_tuned_tile(precision: int, mode: int, n_layer: int, lanes: int, chunk: int, warps: int) -> None:
    st = load_library().socgpu_tune_set(precision, mode, n_layer, lanes, chunk, warps)
    if st != abi.I_NORMAL:
        raise RadianceError(st, "tile not accepted")
