"""Fixture of the reference's CIRC case 6 short-wave known-good output with
the GA7 spectral file, clouds and prescribed soot optical properties.

The reference runs CIRC case 6 (69 layers) in the short wave with the GA7
file, equivalent-extinction gas overlap, continuum, Rayleigh scattering,
delta-rescaling, classic aerosols with the overlay of observed optical
properties, and water and ice clouds of one homogeneous type in a clear and
a cloudy region with maximum-random overlap
(examples/netcdf/CIRC_case6/run_me: Cl_run_cdf -B case6 -s sp_sw_ga7 -R 1 6
-S +R -g 4 -c -r -a +A -C 2 -K 1 -d 5 -i 8, with case6.surfsw_hadgem as
the surface and case6.op_soot_hadgem as the soot optical properties) and
keeps the heating rates in ref_case6_sw_ga7.hrts.  No species has a
mixing-ratio file, so every parametrized species contributes nothing and
soot, overlaid, carries the aerosol.  This script reads the netCDF inputs,
the parsed GA7 short-wave spectral file (block 11 included) and the
reference heating rates from a SOCRATES source tree and stores them in
circ6_sw_ga7.npz beside it (the tree is not available where the tests run
on the GPU).

    python tests/golden/make_circ6_sw.py /path/to/socrates
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
from make_circ6 import SUFFIX, nc_field  # noqa: E402
from socrates_gb300.spectrum import Spectrum  # noqa: E402


def nc_vars(path):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        f = scipy.io.netcdf_file(str(path), "r", mmap=False)
    out = {k: (np.asarray(v[:], dtype=np.float64), v.dimensions) for k, v in f.variables.items()}
    f.close()
    return out


def main(root):
    root = Path(root)
    case = root / "examples" / "netcdf" / "CIRC_case6"
    sp = Spectrum.read_text(root / "data" / "spectra" / "ga7" / "sp_sw_ga7", name="sp_sw_ga7_aer")
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
    arrays = dict(p=p, t=t, p_level=p_level, t_level=t_level, gas=gas, gases_present=np.array(present, np.int32))
    for k in ("szen", "stoa"):
        arrays[k] = nc_field(case / f"case6.{k}", k)[1]
    surf = nc_vars(case / "case6.surfsw_hadgem")
    assert surf["alb"][1][0] == "bands" and surf["alb"][0].shape[1] == 1
    arrays["alb"] = surf["alb"][0][:, 0, 0, 0]                          # one basis function per band
    for k, var in (("clfr", "clfr"), ("lwm", "mixrat"), ("iwm", "mixrat"), ("re", "re"), ("ire", "ire")):
        pk, v = nc_field(case / f"case6.{k}", var)
        assert np.array_equal(pk, p)
        arrays[k] = v
    op = nc_vars(case / "case6.op_soot_hadgem")
    assert op["abs"][1] == ("band", "plev", "lat", "lon") and op["phf"][1] == ("band", "mom", "plev", "lat", "lon")
    arrays["soot_plev"] = op["plev"][0]
    arrays["soot_abs"] = op["abs"][0][:, :, 0, 0]                       # (band, level)
    arrays["soot_scat"] = op["scat"][0][:, :, 0, 0]
    arrays["soot_phf"] = op["phf"][0][:, :, :, 0, 0]                    # (band, moment, level)
    p_out, hrts = field(case / "ref_case6_sw_ga7.hrts")
    assert np.allclose(p_out, p)
    arrays["kgo_hrts"] = hrts
    sp_file = HERE / "_sp_sw_tmp.npz"
    sp.save_npz(sp_file)
    spd = np.load(sp_file)
    arrays.update({"sp_" + k: spd[k] for k in spd.files})
    sp_file.unlink()
    out = HERE / "circ6_sw_ga7.npz"
    np.savez_compressed(out, **arrays)
    print(f"wrote {out} ({out.stat().st_size} bytes); gases with input files: {present}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <SOCRATES source tree>")
    main(sys.argv[1])
