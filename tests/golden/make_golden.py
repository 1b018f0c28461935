"""Regenerate the golden fixtures from the FP64 oracle.

The fixtures pin the oracle's own output (regression), not the reference's:
the reference cannot be compiled here.  Run from the repository root:
    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path[:0] = [str(ROOT), str(ROOT / "oracle"), str(HERE)]

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
from golden_cases import CASES  # noqa: E402


def main():
    for name, case in CASES.items():
        out = case(lambda ctl, sp, col, mc=None: O.radiance_calc(ctl, sp, col, mc))
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
