"""Wen-Yi Zhong's CO2 (band 4) and O3 (band 6) scaling tables as a data file.

The reference compiles these measured tables into its source (the module
scale_wenyi); ip_scale_wenyi needs them at run time.  This library reads
them from a plain text data file instead, which `convert` writes once from a
SOCRATES source tree:

    python -m socrates_gb300.wenyi <path to scale_wenyi.F90> <tables.dat>

The data file (read by `read_data` here and by socgpu_spectrum_load_ext /
socgpu_run -W in C++) is a header line ``socgpu-wenyi-tables 1`` followed by
six arrays, each a line ``<name> <dims...>`` and then its values, whitespace
separated, first index fastest:

    plg 26            ln(p / 100 hPa) grid
    ttb 10            band-4 temperature grid
    tto 9             band-6 temperature grid
    gk250b n4         band-4 normalisation per k-term
    gk4 10 26 n4      band-4 table (temperature, pressure, k-term)
    gk6 9 26 n6       band-6 table (temperature, pressure, k-term)
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

MAGIC = "socgpu-wenyi-tables 1"
_NAMES = ("plg", "ttb", "tto", "gk250b", "gk4", "gk6")


def read_fortran_tables(path) -> dict:
    """The tables from the Fortran source that defines them (the converter's
    input; nothing reads Fortran at run time).  The band-4 and band-6 tables
    are assembled as their RESHAPE(..., ORDER=(3, 2, 1)) builds them: one
    source array per temperature, the k-term index fastest."""
    text = Path(path).read_text()
    arrays = {}
    for m in re.finditer(r"PARAMETER\s*::\s*(\w+)\(\s*(\d+)\s*\)\s*=\s*\(/(.*?)/\)", text, re.S):
        body = re.sub(r"!.*", "", m.group(3))
        vals = [float(v.split("_")[0].replace("D", "E").replace("d", "e"))
                for v in re.findall(r"[-+]?\d+\.?\d*(?:[EeDd][-+]?\d+)?_RealK", body)]
        if len(vals) != int(m.group(2)):
            raise ValueError(f"{path}: {m.group(1)} has {len(vals)} values, declared {m.group(2)}")
        arrays[m.group(1).lower()] = np.array(vals)

    def table(prefix, n_t):
        parts = [arrays[f"{prefix}_{i}"] for i in range(1, n_t + 1)]
        n_term = parts[0].size // 26
        return np.asfortranarray(np.stack([p.reshape(26, n_term) for p in parts], axis=0))

    return dict(wenyi_plg=arrays["plg"], wenyi_ttb=arrays["ttb"], wenyi_tto=arrays["tto"],
                wenyi_gk250b=arrays["gk250b"], wenyi_gk4=table("gk4", arrays["ttb"].size),
                wenyi_gk6=table("gk6", arrays["tto"].size))


def write_data(path, tables: dict) -> None:
    """Write the tables (keys wenyi_plg ... wenyi_gk6) as the data file."""
    lines = [MAGIC]
    for name in _NAMES:
        a = np.asarray(tables["wenyi_" + name], dtype=np.float64)
        lines.append(name + " " + " ".join(str(d) for d in a.shape))
        flat = a.reshape(-1, order="F")
        for q in range(0, flat.size, 6):
            lines.append(" ".join(f"{v:.17e}" for v in flat[q:q + 6]))
    Path(path).write_text("\n".join(lines) + "\n")


def read_data(path) -> dict:
    """Read the data file; returns the keys wenyi_plg ... wenyi_gk6."""
    tok = Path(path).read_text().split()
    if " ".join(tok[:2]) != MAGIC:
        raise ValueError(f"{path}: not a Wen-Yi tables file (no '{MAGIC}' header)")
    pos, out = 2, {}
    ndim = {"plg": 1, "ttb": 1, "tto": 1, "gk250b": 1, "gk4": 3, "gk6": 3}
    for name in _NAMES:
        if pos >= len(tok) or tok[pos] != name:
            raise ValueError(f"{path}: expected the array '{name}'")
        shape = tuple(int(t) for t in tok[pos + 1:pos + 1 + ndim[name]])
        pos += 1 + ndim[name]
        n = int(np.prod(shape))
        vals = np.array([float(t) for t in tok[pos:pos + n]])
        if vals.size != n:
            raise ValueError(f"{path}: '{name}' is short of values")
        pos += n
        out["wenyi_" + name] = np.asfortranarray(vals.reshape(shape, order="F"))
    return out


def convert(source, out) -> None:
    write_data(out, read_fortran_tables(source))


if __name__ == "__main__":
    if len(sys.argv) != 3:
        sys.exit("usage: python -m socrates_gb300.wenyi <scale_wenyi.F90> <tables.dat>")
    convert(sys.argv[1], sys.argv[2])
