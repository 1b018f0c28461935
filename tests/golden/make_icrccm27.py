"""Fixture of the reference's ICRCCM case 27 known-good output.

The reference tests its infra-red code on ICRCCM case 27 (AER profile, 60
layers) with the HadCM3 spectral file, random gas overlap, water-vapour
continuum, Elsasser two-stream, solver 13 and clear sky
(examples/aer_cmp/run27: Cl_run_cdl -s sp_lw_hadcm3 -R 1 8 -I -g 2 -c -t 12
-v 13 -C 5), and compares the heating rates with laer27_ref.hrts.  This
script reads those inputs, the parsed spectral file and the reference
heating rates from a SOCRATES source tree and stores them in
icrccm27_lw_hadcm3.npz beside it (the tree is not available where the tests
run on the GPU).

    python tests/golden/make_icrccm27.py /path/to/socrates
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE))

from cdl import field  # noqa: E402
from socrates_gb300.spectrum import Spectrum  # noqa: E402

SUFFIX = {1: "q", 2: "co2", 3: "o3", 4: "n2o", 6: "ch4", 14: "cfc11", 15: "cfc12", 16: "cfc113", 17: "hcfc22",
          18: "hfc125", 19: "hfc134a"}


def main(root):
    root = Path(root)
    case = root / "examples" / "aer_cmp"
    sp = Spectrum.read_text(root / "data" / "spectra" / "hadcm3" / "sp_lw_hadcm3", name="sp_lw_hadcm3")
    p, t = field(case / "laer27.t")
    p_level, t_level = field(case / "laer27.tl")
    gas = np.zeros((p.size, sp.n_absorb))
    for j, ty in enumerate(sp.type_absorb):
        pg, v = field(case / f"laer27.{SUFFIX[int(ty)]}")
        assert np.array_equal(pg, p), f"{SUFFIX[int(ty)]} is not on the temperature grid"
        gas[:, j] = v
    _, tstar = field(case / "laer27.tstar")
    _, alb = field(case / "laer27.surf", coord="basis")
    p_out, hrts = field(case / "laer27_ref.hrts")
    assert np.allclose(p_out, p)
    out = HERE / "icrccm27_lw_hadcm3.npz"
    arrays = dict(p=p, t=t, p_level=p_level, t_level=t_level, gas=gas, t_ground=tstar, alb=alb, kgo_hrts=hrts)
    sp_file = HERE / "_sp_tmp.npz"
    sp.save_npz(sp_file)
    spd = np.load(sp_file)
    arrays.update({"sp_" + k: spd[k] for k in spd.files})
    sp_file.unlink()
    np.savez_compressed(out, **arrays)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <SOCRATES source tree>")
    main(sys.argv[1])
