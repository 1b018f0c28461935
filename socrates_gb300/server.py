"""Continuous-batching request server over the C-ABI (socgpu_server_*).

A request is a radiance_calc call with host arrays (a Marshal).  submit()
returns at once with a ticket.  The library's scheduler thread admits
requests by free device memory and runs them in overlapping waves.  wait()
returns the request's status and its latencies.  The Marshal's arrays
(inputs and outputs) must stay alive until wait() returns.
"""
from __future__ import annotations

import ctypes as C

from . import abi
from .radiance import Marshal, RadianceError, load_library, register_spectrum


class Server:
    def __init__(self, device_bytes: int = 0, streams: int = 4, max_wave_requests: int = 256,
                 small_column_gpoints: int = 0):
        self.lib = load_library()
        cfg = abi.ServerConfig(device_bytes, streams, max_wave_requests, small_column_gpoints)
        self.handle = C.c_void_p()
        msg = C.create_string_buffer(512)
        st = self.lib.socgpu_server_create(C.byref(cfg), C.byref(self.handle), msg, 512)
        if st != abi.I_NORMAL:
            raise RadianceError(st, msg.value.decode())
        self._held: dict[int, tuple] = {}

    def submit(self, m: Marshal, spectrum) -> int:
        item = abi.BatchItem(C.pointer(m.control), C.pointer(m.dimen), register_spectrum(spectrum), C.pointer(m.atm),
                             C.pointer(m.cld), C.pointer(m.aer), C.pointer(m.bound), C.pointer(m.radout))
        t = C.c_longlong()
        msg = C.create_string_buffer(512)
        st = self.lib.socgpu_server_submit(self.handle, C.byref(item), C.byref(t), msg, 512)
        if st != abi.I_NORMAL:
            raise RadianceError(st, msg.value.decode())
        self._held[t.value] = (m, item)
        return t.value

    def wait(self, ticket: int, timeout_s: float = -1.0) -> tuple[float, float]:
        """Block until the request is done; returns (queue ms, latency ms)."""
        status, q, lat = C.c_int(), C.c_double(), C.c_double()
        msg = C.create_string_buffer(512)
        st = self.lib.socgpu_server_wait(self.handle, ticket, timeout_s, C.byref(status), C.byref(q), C.byref(lat),
                                         msg, 512)
        if st != abi.I_NORMAL:
            raise RadianceError(st, msg.value.decode())
        self._held.pop(ticket, None)
        if status.value != abi.I_NORMAL:
            raise RadianceError(status.value, msg.value.decode())
        return q.value, lat.value

    def stats(self) -> dict:
        s = abi.ServerStats()
        self.lib.socgpu_server_stats_get(self.handle, C.byref(s))
        return {k: getattr(s, k) for k, _ in abi.ServerStats._fields_}

    def close(self) -> None:
        if self.handle:
            self.lib.socgpu_server_destroy(self.handle)
            self.handle = C.c_void_p()
            self._held.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
