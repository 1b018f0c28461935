"""Build the FP64 CPU oracle (test infrastructure only).

Compiles ``oracle/socrates_oracle.c`` into ``oracle/_build/liboracle.so``
with OpenMP and without floating-point contraction, so its FP64 results
follow the reference's operation order on both x86-64 and aarch64.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "socrates_oracle.c"
OUT = HERE / "_build" / "liboracle.so"
INCLUDE = HERE.parent / "include"


def build(force: bool = False) -> Path:
    deps = [SRC, HERE / "socrates_oracle.h", INCLUDE / "socgpu.h", Path(__file__)]
    if not force and OUT.exists() and all(OUT.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           f"-I{INCLUDE}", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
