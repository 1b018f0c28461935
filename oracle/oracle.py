"""Python entry to the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, the smoke check and bench.py's CPU-baseline leg as the
checker.  It feeds the oracle the same C structures the product library
receives (socrates_gb300.radiance.Marshal), so both see identical inputs.
The restatement is pinned to the reference's printed known-good outputs
(ICRCCM case 27, CIRC case 6, the runes test, the McICA and cloud-region
examples): see socrates_oracle.h.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

from socrates_gb300 import abi  # noqa: E402
from socrates_gb300.radiance import Marshal, McicaState, RadianceError  # noqa: E402

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("oracle_build", HERE / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        lib = C.CDLL(str(mod.build()))
        calc = [C.POINTER(abi.Control), C.POINTER(abi.Dimen), C.POINTER(abi.SpectrumDesc), C.POINTER(abi.Atm),
                C.POINTER(abi.Cld), C.POINTER(abi.Aer), C.POINTER(abi.Bound), C.POINTER(abi.Radout)]
        lib.oracle_radiance_calc.argtypes = calc + [C.c_char_p, C.c_size_t]
        lib.oracle_radiance_calc.restype = C.c_int
        lib.oracle_radiance_calc_segmented.argtypes = calc + [C.c_int, C.c_char_p, C.c_size_t]
        lib.oracle_radiance_calc_segmented.restype = C.c_int
        lib.oracle_cloud_gen.argtypes = [C.c_int] * 11 + [C.c_void_p] * 9 + [C.c_void_p, C.c_void_p, C.c_int]
        lib.oracle_cloud_gen.restype = C.c_int
        lib.oracle_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        _lib = lib
    return _lib


def radiance_calc(control, spectrum, col, mcica: McicaState | None = None, id_cloud_top: int = 1,
                  threads: int = 1) -> dict:
    lib = load()
    m = Marshal(control, spectrum, col, mcica, id_cloud_top)
    desc = spectrum.to_desc()
    msg = C.create_string_buffer(512)
    if threads == 1:
        st = lib.oracle_radiance_calc(*m.args(C.byref(desc)), msg, 512)
    else:
        st = lib.oracle_radiance_calc_segmented(*m.args(C.byref(desc)), threads, msg, 512)
    if st != abi.I_NORMAL:
        raise RadianceError(st, msg.value.decode())
    return m.result()


def cloud_gen_impl(*args):
    return load().oracle_cloud_gen(*args)


def philox(ctr, key):
    lib = load()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib.oracle_philox4x32_10(c, k, o)
    return list(o)
