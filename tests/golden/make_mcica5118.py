"""Fixture of the reference's McICA known-good outputs (examples/netcdf/mcica):
one 52-layer column of cloud-resolving-model data, 5118_142, run with McICA
(-C 10), clouds as one homogeneous type of water and ice (-K 1), the
relative standard deviation of condensate 0.75 (-m), optimal sampling (+m 2)
and a decorrelation pressure scale of 10000 Pa (-dp), with rescaling (+R):

    lw_avg     sp_lw_ga3_0  -R 1 9 -I -t 12 -v 13 -g 5 -c -d 1 -i 1
    sw_avg     sp_sw_ga3_0  -R 1 6 -S -t 2  -v 13 -g 5 -r -d 3 -i 3
    sw_ds0_avg sp_sw_ga3_0  as sw_avg, direct beam not delta-scaled (-ds 0)
    lw_ga7     sp_lw_ga7    -R 1 9 -I -g 4 -c -d 5 -i 8
    sw_ga7     sp_sw_ga7    -R 1 6 -S -g 4 -r -d 5 -i 8

The known-good heating rates are ref_<run>.hrts (6 significant digits).
This script reads the netCDF inputs, the GA3.0 spectral files (the GA7 ones
are in circ6_lw_ga7.npz and ga7_sw_spectrum.npz), both McICA data files and
the known-good outputs from a SOCRATES source tree, and stores them in
mcica5118.npz beside it.  cloud_gen reads the water-content table xcw only
in the columns next to 40 sigma - 3 = 27 (socrates_cloud_gen.F90:313-323), so
the fixture keeps columns 20-35 of it.

    python tests/golden/make_mcica5118.py /path/to/socrates
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE))

from cdl import field  # noqa: E402
from make_circ6 import nc_field  # noqa: E402
from socrates_gb300.radiance import read_mcica_data  # noqa: E402
from socrates_gb300.spectrum import Spectrum  # noqa: E402
from socrates_gb300.wenyi import read_fortran_tables  # noqa: E402

RUNS = ("lw_avg", "sw_avg", "sw_ds0_avg", "lw_ga7", "sw_ga7")
FIELDS = ("q", "co2", "o3", "n2o", "ch4", "o2", "clfr", "lwm", "iwm", "re", "ire")
XCW_COLS = (20, 36)        # 1-based columns 20..35


def main(root):
    root = Path(root)
    case = root / "examples" / "netcdf" / "mcica"
    arrays = {}
    p, t = nc_field(case / "5118_142.t", "t")
    p_level, t_level = nc_field(case / "5118_142.tl", "tl")
    arrays.update(p=p, t=t, p_level=p_level, t_level=t_level)
    for name in FIELDS:
        pg, v = nc_field(case / f"5118_142.{name}", name)
        assert np.array_equal(pg, p), name
        arrays[name] = v
    for name, var in (("tstar", "tstar"), ("szen", "szen"), ("stoa", "stoa"), ("surflw", "alb"), ("surfsw", "alb")):
        arrays[name] = nc_field(case / f"5118_142.{name}", var)[1]
    for run in RUNS:
        pk, hr = field(case / f"ref_{run}.hrts")
        assert np.allclose(pk, p)
        arrays["kgo_" + run] = hr
    wy = read_fortran_tables(root / "src" / "radiance_core" / "scale_wenyi.F90")
    for pre, name in (("lw_", "sp_lw_ga3_0"), ("sw_", "sp_sw_ga3_0")):
        sp = Spectrum.read_text(root / "data" / "spectra" / "ga3_0" / name, name=name)
        if pre == "lw_":
            for k, v in wy.items():
                setattr(sp, k, v)
        tmp = HERE / "_sp_tmp.npz"
        sp.save_npz(tmp)
        spd = np.load(tmp)
        arrays.update({pre + k: spd[k] for k in spd.files})
        tmp.unlink()
    c0, c1 = XCW_COLS
    for pre, sub in (("ga3_", "ga3_0"), ("ga7_", "ga7")):
        d = read_mcica_data(root / "data" / "spectra" / sub / "mcica_data")
        arrays[pre + "scalars"] = np.array([d.n_subcol_gen, d.n_subcol_req_single, d.n_subcol_req_optimal, d.ipph,
                                            d.xcw.shape[0], d.xcw.shape[1], c0, c1], np.int32)
        arrays[pre + "reorder_single"] = d.lw_subcol_reorder_single
        arrays[pre + "reorder_optimal"] = d.lw_subcol_reorder_optimal
        for key in ("sw_subcol_k", "lw_subcol_k"):
            tab = getattr(d, key) or {}
            arrays[pre + key] = np.array([[b, k, n] for (b, k), n in sorted(tab.items())], np.int32).reshape(-1, 3)
        arrays[pre + "xcw_cols"] = np.asfortranarray(d.xcw[:, c0 - 1:c1 - 1])
    out = HERE / "mcica5118.npz"
    np.savez_compressed(out, **arrays)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <SOCRATES source tree>")
    main(sys.argv[1])
