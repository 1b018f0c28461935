"""Fixture of the reference's CIRC case 6 clear-sky long-wave known-good output
with the GA7 spectral file.

The reference runs CIRC case 6 (69 layers) with the GA7 long-wave spectral
file, equivalent-extinction gas overlap, water-vapour continuum and clear sky
(examples/netcdf/CIRC_case6/run_me: Cl_run_cdf -B case6 -s sp_lw_ga7 -R 1 9
-I -g 4 -c -C 5) and keeps the heating rates in ref_case6_lw_ga7_clr.hrts.
GA7 takes most of its k-terms from the lookup tables of sp_lw_ga7_k and the
CO2 terms of band 4 from Wen-Yi Zhong's tables (module scale_wenyi).  This
script reads the netCDF inputs, the parsed spectral file with its tables and
the reference heating rates from a SOCRATES source tree and stores them in
circ6_lw_ga7.npz beside it, and the parsed GA7 short-wave spectral file in
ga7_sw_spectrum.npz (the tree is not available where the tests run on the
GPU).  Absorbers without an input file (SO2, CFC113, HCFC22, HFC134a,
OCS) have zero mixing ratios, as l_run_cdf.F90:797-833 sets them.

    python tests/golden/make_circ6.py /path/to/socrates
"""
import sys
import warnings
from pathlib import Path

import numpy as np
import scipy.io

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE))

from cdl import field  # noqa: E402
from socrates_gb300.spectrum import Spectrum  # noqa: E402
from socrates_gb300.wenyi import read_fortran_tables  # noqa: E402

# file suffixes of the gases (input_head_pcf.f90:208-225)
SUFFIX = {1: "q", 2: "co2", 3: "o3", 4: "n2o", 6: "ch4", 7: "o2", 9: "so2", 14: "cfc11", 15: "cfc12",
          16: "cfc113", 17: "hcfc22", 19: "hfc134a", 25: "ocs"}


def nc_field(path, name):
    """(coordinate, values) of a one-profile netCDF input file, in FP64."""
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        f = scipy.io.netcdf_file(str(path), "r", mmap=False)
    v = np.asarray(f.variables[name][:], dtype=np.float64).ravel()
    coord = np.asarray(f.variables["plev"][:], dtype=np.float64) if "plev" in f.variables else None
    f.close()
    return coord, v


def main(root):
    root = Path(root)
    case = root / "examples" / "netcdf" / "CIRC_case6"
    sp = Spectrum.read_text(root / "data" / "spectra" / "ga7" / "sp_lw_ga7", name="sp_lw_ga7")
    for k, v in read_fortran_tables(root / "src" / "radiance_core" / "scale_wenyi.F90").items():
        setattr(sp, k, v)
    p, t = nc_field(case / "case6.t", "t")
    p_level, t_level = nc_field(case / "case6.tl", "tl")
    gas = np.zeros((p.size, sp.n_absorb))
    present = []
    for j, ty in enumerate(sp.type_absorb):
        f = case / f"case6.{SUFFIX[int(ty)]}"
        if not f.exists():
            continue
        pg, v = nc_field(f, SUFFIX[int(ty)])
        assert np.array_equal(pg, p), f"{f.name} is not on the temperature grid"
        gas[:, j] = v
        present.append(int(ty))
    _, tstar = nc_field(case / "case6.tstar", "tstar")
    _, alb = nc_field(case / "case6.surflw", "alb")
    p_out, hrts = field(case / "ref_case6_lw_ga7_clr.hrts")
    assert np.allclose(p_out, p)
    out = HERE / "circ6_lw_ga7.npz"
    arrays = dict(p=p, t=t, p_level=p_level, t_level=t_level, gas=gas, t_ground=tstar, alb=alb, kgo_hrts=hrts,
                  gases_present=np.array(present, np.int32))
    sp_file = HERE / "_sp_tmp.npz"
    sp.save_npz(sp_file)
    spd = np.load(sp_file)
    arrays.update({"sp_" + k: spd[k] for k in spd.files})
    sp_file.unlink()
    np.savez_compressed(out, **arrays)
    print(f"wrote {out} ({out.stat().st_size} bytes); gases with input files: {present}")
    # the GA7 short-wave spectral file (lookup tables, no Wen-Yi terms), for
    # synthetic solar cases
    sw = Spectrum.read_text(root / "data" / "spectra" / "ga7" / "sp_sw_ga7", name="sp_sw_ga7")
    sw_out = HERE / "ga7_sw_spectrum.npz"
    sw.save_npz(sw_out)
    print(f"wrote {sw_out} ({sw_out.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <SOCRATES source tree>")
    main(sys.argv[1])
