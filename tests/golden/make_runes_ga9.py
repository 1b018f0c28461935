"""Fixture of the reference's runes test (examples/runes/run_me): the driver
src/aux/runes_driver.f90 calls runes on a 32-layer mid-latitude summer
profile with the GA9 spectral files, clear sky: a solar call with Rayleigh
scattering, then three thermal calls with the surface given by its skin
temperature, by its emission per band, and by two tiles (one with its
emission given, one with its temperature).  The known-good output
(examples/runes/gfortran_8_1_0.txt) lists, for levels 1..32, the downward
and upward fluxes and the layer heating rates in K/day.

The driver's literals are default-real (single precision) constants assigned
to RealExt (double precision) variables, and its pi is 4 atan(1) in single
precision: the fixture keeps those values.  This script reads the driver,
the GA9 spectral files with their '_k' tables, the Wen-Yi tables and the
known-good output from a SOCRATES source tree and stores them in
runes_ga9.npz beside it.

    python tests/golden/make_runes_ga9.py /path/to/socrates
"""
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from socrates_gb300.spectrum import Spectrum  # noqa: E402
from socrates_gb300.wenyi import read_fortran_tables  # noqa: E402


def single(x):
    """A default-real literal as the compiler stores it."""
    return np.float64(np.float32(x))


def driver_data(text):
    """The data statements of runes_driver.f90: arrays and scalars."""
    out = {}
    for m in re.finditer(r"real\(RealExt\)(?:, target)? :: (\w+)(\([^)]*\))? = reshape\( \(/(.*?)/\)", text, re.S):
        vals = [single(v) for v in re.findall(r"[-+]?\d+\.\d*(?:[Ee][-+]?\d+)?", re.sub(r"!.*", "", m.group(3)))]
        out[m.group(1)] = np.array(vals)
    for m in re.finditer(r"real\(RealExt\)(?:, parameter)? :: (\w+)(\([^)]*\))? = ([-+]?\d+\.?\d*(?:[Ee][-+]?\d+)?)\s*$",
                         text, re.M):
        out[m.group(1)] = single(m.group(3))
    m = re.search(r"logical :: l_flux_tile\(n_tile\) = \(/(.*?)/\)", text)
    out["l_flux_tile"] = np.array([v.strip().lower() == ".true." for v in m.group(1).split(",")], np.int32)
    return out


def kgo(text):
    """The four sections of the known-good output, each (32, 3)."""
    sections, cur = [], None
    for ln in text.splitlines():
        if "flux down" in ln:
            cur = []
            sections.append(cur)
        elif cur is not None and ln.strip() and re.match(r"^\s*[-\d.]+\s+[-\d.]+\s+[-\d.]+\s*$", ln):
            cur.append([float(x) for x in ln.split()])
    return [np.array(s) for s in sections]


def main(root):
    root = Path(root)
    d = driver_data((root / "src" / "aux" / "runes_driver.f90").read_text())
    pi = np.float64(np.float32(4.0) * np.arctan(np.float32(1.0)))
    cos_zen = np.cos(45.0 * pi / 180.0)
    sections = kgo((root / "examples" / "runes" / "gfortran_8_1_0.txt").read_text())
    assert len(sections) == 4 and all(s.shape == (32, 3) for s in sections)
    sw = Spectrum.read_text(root / "data" / "spectra" / "ga9" / "sp_sw_ga9", name="sw")
    lw = Spectrum.read_text(root / "data" / "spectra" / "ga9" / "sp_lw_ga9", name="lw")
    for k, v in read_fortran_tables(root / "src" / "radiance_core" / "scale_wenyi.F90").items():
        setattr(lw, k, v)
    arrays = dict(cos_zenith_angle=np.array([cos_zen]), kgo_sw=sections[0], kgo_lw_tground=sections[1],
                  kgo_lw_flux_ground=sections[2], kgo_lw_tiles=sections[3])
    for k in ("p_layer", "t_layer", "p_level", "t_level", "h2o", "o3", "flux_ground", "flux_tile", "frac_tile"):
        arrays[k] = d[k]
    for k in ("grav_acc", "r_gas_dry", "cp_air_dry", "t_ground", "co2_mix_ratio", "ch4_mix_ratio", "n2o_mix_ratio",
              "o2_mix_ratio", "solar_irrad", "grey_albedo_sw", "grey_albedo_lw", "t_tile"):
        arrays[k] = np.array(d[k])
    arrays["l_flux_tile"] = d["l_flux_tile"]
    for prefix, sp in (("sw_", sw), ("lw_", lw)):
        tmp = HERE / "_sp_tmp.npz"
        sp.save_npz(tmp)
        spd = np.load(tmp)
        arrays.update({prefix + k: spd[k] for k in spd.files})
        tmp.unlink()
    out = HERE / "runes_ga9.npz"
    np.savez_compressed(out, **arrays)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <SOCRATES source tree>")
    main(sys.argv[1])
