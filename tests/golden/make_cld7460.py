"""Fixture of the reference's cloud-region known-good outputs
(examples/netcdf/7460_28): 167 layers of cloud-resolving-model data, as their
average (one column) and as 20 columns (ipa0/), with clouds in a clear and a
cloudy region of maximum-random overlap (-C 2) and water and ice as one
homogeneous cloud type (-K 1):

    lw_avg      sp_lw_hadgem1_3  -R 1 9 -I -t 12 +R -v 11 -g 2 -c -d 1 -i 1   (.surflw)
    sw_avg      sp_sw_hadgem1_3  -R 1 6 -S -t 2 +R -v 11 -g 2 -r -d 3 -i 3    (.surfsw)
    sw_ds0_avg  as sw_avg, direct beam not delta-scaled (-ds 0)
    sw2         as sw_avg with .surfsw2 (diffuse and direct albedos)
    sw2_ds0     as sw2 with -ds 0
    sw_ga9_avg  sp_sw_ga9  -R 1 6 -S +R -g 4 -c -r -d 5 -i 8  (solver 16)   (.surfsw2)
    lw_ga9_avg  sp_lw_ga9  -R 1 9 -I +R -g 4 -c -d 5 -i 8     (solver 16)   (.surflw)
    ipa_lw, ipa_sw  the first two on the 20 columns

The known-good outputs are ref_<run>.hrts (6 significant digits), or the
net fluxes ref_<run>.nflx where only those are kept.  This script reads the
inputs, the HadGEM1 spectral files and the known-good outputs from a SOCRATES
source tree and stores them in cld7460.npz beside it (the GA9 files are in
runes_ga9.npz).

    python tests/golden/make_cld7460.py /path/to/socrates
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

LAYER_FIELDS = ("t", "q", "co2", "o3", "n2o", "ch4", "o2", "clfr", "lwm", "iwm", "re", "ire")
KGO = {"lw_avg": "ref_lw_avg.hrts", "sw_avg": "ref_sw_avg.hrts", "sw_ds0_avg": "ref_sw_ds0_avg.hrts",
       "sw2": "ref_sw2.hrts", "sw2_ds0": "ref_sw2_ds0.hrts", "sw_ga9_avg": "ref_sw_ga9_avg.nflx",
       "lw_ga9_avg": "ref_lw_ga9_avg.nflx"}


def nc(path):
    """(plev or None, data as (levels, columns)) of a netCDF column file."""
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        f = scipy.io.netcdf_file(str(path), "r", mmap=False)
    var = next(v for k, v in f.variables.items() if k not in ("lat", "lon", "plev", "basis", "band"))
    a = np.asarray(var[:], dtype=np.float64)
    coord = np.asarray(f.variables["plev"][:], dtype=np.float64) if "plev" in f.variables else None
    f.close()
    return coord, a.reshape(a.shape[0], -1) if a.ndim > 1 else a.reshape(1, -1)


def main(root):
    root = Path(root)
    case = root / "examples" / "netcdf" / "7460_28"
    arrays = {}
    for pre, d in (("avg_", case), ("ipa_", case / "ipa0")):
        p, t = nc(d / "7460_28.t")
        pl, tl = nc(d / "7460_28.tl")
        arrays.update({pre + "p": p, pre + "p_level": pl, pre + "t_level": tl})
        for name in LAYER_FIELDS:
            pg, v = nc(d / f"7460_28.{name}")
            assert np.array_equal(pg, p), name
            arrays[pre + name] = v
        for name in ("tstar", "szen", "stoa", "surflw", "surfsw"):
            arrays[pre + name] = nc(d / f"7460_28.{name}")[1].ravel()
    arrays["avg_surfsw2"] = nc(case / "7460_28.surfsw2")[1].ravel()
    for run, fname in KGO.items():
        pk, v = field(case / fname)
        arrays["kgo_" + run] = v
    for run in ("lw", "sw"):
        arrays[f"kgo_ipa_{run}"] = nc(case / "ipa0" / f"ref_{run}.hrts")[1]
    for pre, name in (("hlw_", "sp_lw_hadgem1_3"), ("hsw_", "sp_sw_hadgem1_3")):
        sp = Spectrum.read_text(root / "data" / "spectra" / "hadgem1" / name, name=name)
        tmp = HERE / "_sp_tmp.npz"
        sp.save_npz(tmp)
        spd = np.load(tmp)
        arrays.update({pre + k: spd[k] for k in spd.files})
        tmp.unlink()
    out = HERE / "cld7460.npz"
    np.savez_compressed(out, **arrays)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <SOCRATES source tree>")
    main(sys.argv[1])
