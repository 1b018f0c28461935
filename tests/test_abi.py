"""CPU checks of the C-ABI library: it builds, loads without a GPU and
exports every entry point include/socgpu.h declares; host-only argument
validation answers with the reference's error codes."""
import ctypes as C
from pathlib import Path

import pytest

from socrates_gb300 import abi, build
from socrates_gb300.spectrum import Spectrum
from socrates_gb300 import synth

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    path = build.build()
    return abi.declare(C.CDLL(str(path)))


def test_every_declared_symbol_is_exported(lib):
    names = abi.header_functions(ROOT / "include" / "socgpu.h")
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(abi.ABI_FUNCTIONS)


def test_abi_version(lib):
    assert lib.socgpu_abi_version() == abi.ABI_VERSION


def test_tile_config_validation(lib):
    assert lib.socgpu_set_tile_config(abi.PRECISION_MIXED, 1, 8, 4) == abi.I_NORMAL
    assert lib.socgpu_set_tile_config(abi.PRECISION_FP64, 1, 8, 4) == abi.I_ERR_RANGE
    assert lib.socgpu_set_tile_config(abi.PRECISION_MIXED, 3, 8, 4) == abi.I_ERR_RANGE
    assert lib.socgpu_set_tile_config(abi.PRECISION_MIXED, 1, 12, 4) == abi.I_ERR_RANGE
    assert lib.socgpu_set_tile_config(abi.PRECISION_MIXED, 1, 0, 0) == abi.I_NORMAL


def test_lookup_of_unknown_spectrum(lib):
    h = C.c_int(0)
    assert lib.socgpu_spectrum_lookup(b"no-such-spectrum", C.byref(h)) == abi.I_ERR_EXIST


def test_spectral_file_round_trip(tmp_path):
    for sp in (synth.lw_spectrum(1, 9, clouds=True), synth.sw_spectrum(2, 8, clouds=True)):
        path = tmp_path / "sp"
        sp.write_text(path)
        back = Spectrum.read_text(path)
        assert back.n_band == sp.n_band and back.n_gpoint == sp.n_gpoint
        for name in ("k", "w", "p_ref", "t_ref", "i_band_k", "i_scale_fnc", "index_absorb"):
            a, b = getattr(sp, name), getattr(back, name)
            assert a.shape == b.shape and (abs(a - b) <= 1e-9 * abs(a) + 1e-300).all(), name
        if sp.thermal_coeff is not None:
            assert abs(back.thermal_coeff - sp.thermal_coeff).max() <= 1e-8 * abs(sp.thermal_coeff).max()
        if sp.solar_flux_band is not None:
            assert abs(back.solar_flux_band - sp.solar_flux_band).max() < 1e-9
        if sp.rayleigh_coeff is not None:
            # every band, the first included (block 3 has three header records)
            assert (abs(back.rayleigh_coeff - sp.rayleigh_coeff) <= 1e-9 * sp.rayleigh_coeff).all()
        # cloud parameter sets are written as read_block_10_0_2 reads them,
        # 4(4x, 1pe12.5): six significant digits
        for a, b in ((sp.drop_parm_list, back.drop_parm_list), (sp.ice_parm_list, back.ice_parm_list)):
            assert a.shape == b.shape and (abs(a - b) <= 5.0e-6 * abs(a)).all()
        assert (back.i_drop_parm == sp.i_drop_parm).all() and (back.i_ice_parm == sp.i_ice_parm).all()


def test_tile_table_validation(lib):
    # host-only bookkeeping: no device call
    assert lib.socgpu_tune_set(1, 1, 100, 32, 4, 8) == abi.I_NORMAL
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    assert lib.socgpu_tune_get(1, 1, 100, C.byref(a), C.byref(b), C.byref(c)) == abi.I_NORMAL
    assert (a.value, b.value, c.value) == (32, 4, 8)
    assert lib.socgpu_tune_set(1, 1, 100, 32, 3, 8) == abi.I_ERR_RANGE     # 96 layers do not cover 100
    assert lib.socgpu_tune_set(1, 1, 100, 32, 6, 8) == abi.I_ERR_RANGE     # no 6-layer chunk is built
    assert lib.socgpu_tune_set(0, 1, 100, 8, 13, 8) == abi.I_ERR_RANGE     # FP64 has no 8-lane kernels
    assert lib.socgpu_tune_set(1, 1, 100, 0, 0, 0) == abi.I_NORMAL          # remove
    assert lib.socgpu_tune_get(1, 1, 100, C.byref(a), C.byref(b), C.byref(c)) == abi.I_ERR_EXIST


def test_ctypes_structs_match_the_header(tmp_path):
    """Every ctypes mirror in abi.py has the size and field offsets of its
    struct in include/socgpu.h, as gcc lays them out."""
    import ctypes as C
    import subprocess
    from pathlib import Path
    from socrates_gb300 import abi
    root = Path(__file__).resolve().parent.parent
    mirrors = {"socgpu_spectrum_desc": abi.SpectrumDesc, "socgpu_control": abi.Control, "socgpu_dimen": abi.Dimen,
               "socgpu_atm": abi.Atm, "socgpu_bound": abi.Bound, "socgpu_aer": abi.Aer, "socgpu_cld": abi.Cld,
               "socgpu_radout": abi.Radout, "socgpu_runes_args": abi.RunesArgs, "socgpu_runes_diag": abi.RunesDiag,
               "socgpu_batch_item": abi.BatchItem, "socgpu_server_config": abi.ServerConfig,
               "socgpu_server_stats": abi.ServerStats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "socgpu.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{root / 'include'}", str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        cname, field, value = ln.split()
        got[(cname, field)] = int(value)
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, f"{cname}.{fname}"
