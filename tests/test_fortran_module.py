"""include/socgpu_mod.f90 against the C structs of include/socgpu.h.

No Fortran compiler is available here, so the module is checked as text:
every BIND(C) derived type must list the members of its C struct (the
ctypes mirrors in socrates_gb300/abi.py, whose layouts test_abi checks
against the header), in the same order and with interoperable kinds, and
every interface must bind a function the library exports.
"""
import ctypes as C
import re
from pathlib import Path

from socrates_gb300 import abi

ROOT = Path(__file__).resolve().parent.parent
MOD = ROOT / "include" / "socgpu_mod.f90"

MIRRORS = {"socgpu_control": abi.Control, "socgpu_dimen": abi.Dimen, "socgpu_atm": abi.Atm,
           "socgpu_bound": abi.Bound, "socgpu_aer": abi.Aer, "socgpu_cld": abi.Cld, "socgpu_radout": abi.Radout,
           "socgpu_runes_args": abi.RunesArgs, "socgpu_runes_diag": abi.RunesDiag}
KIND = {"c_int": C.c_int, "c_double": C.c_double, "c_ptr": C.c_void_p}


def _fortran_types(text):
    """{type name: [(member, kind, count)]} of the BIND(C) derived types."""
    params = {m.group(1).lower(): int(m.group(2))
              for m in re.finditer(r"INTEGER,\s*PARAMETER\s*::\s*(\w+)\s*=\s*(\d+)", text)}
    out = {}
    for m in re.finditer(r"TYPE,\s*BIND\(C\)\s*::\s*(\w+)(.*?)END TYPE", text, re.S):
        members = []
        body = re.sub(r"&\s*\n\s*", " ", m.group(2))
        for line in body.splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            d = re.match(r"(INTEGER|REAL|TYPE)\((c_\w+)\)\s*::\s*(.*)", line)
            assert d, f"unparsed member line in {m.group(1)}: {line}"
            kind = d.group(2)
            for item in re.findall(r"(\w+)(?:\((\w+)\))?", d.group(3)):
                name, dim = item
                count = 1 if not dim else (int(dim) if dim.isdigit() else params[dim.lower()])
                members.append((name.lower(), kind, count))
        out[m.group(1).lower()] = members
    return out


def _ctype_fields(py):
    out = []
    for name, t in py._fields_:
        count = 1
        if issubclass(t, C.Array):
            count, t = t._length_, t._type_
        if issubclass(t, C._Pointer) or t in (C.c_void_p, C.c_char_p):
            kind = C.c_void_p
        else:
            kind = t
        out.append((name.lower(), kind, count))
    return out


def test_fortran_types_mirror_the_c_structs():
    types = _fortran_types(MOD.read_text())
    assert set(MIRRORS) <= set(types), set(MIRRORS) - set(types)
    for name, py in MIRRORS.items():
        f = types[name]
        c = _ctype_fields(py)
        assert [m[0] for m in f] == [m[0] for m in c], f"{name}: member names or order differ"
        for (mn, fk, fc), (_, ck, cc) in zip(f, c):
            assert KIND[fk] == ck or (fk == "c_int" and ck in (C.c_int, C.c_int32)), f"{name}.{mn}: {fk} vs {ck}"
            assert fc == cc, f"{name}.{mn}: {fc} elements vs {cc}"


def test_fortran_interfaces_bind_exported_functions():
    text = MOD.read_text()
    names = re.findall(r"BIND\(C,\s*NAME='(\w+)'\)", text)
    assert "socgpu_radiance_calc" in names and "socgpu_runes" in names
    assert set(names) <= set(abi.ABI_FUNCTIONS), set(names) - set(abi.ABI_FUNCTIONS)
