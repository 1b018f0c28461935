"""Build libsocgpu.so in-tree for sm_103a.

Each translation unit under csrc/ is compiled by its own nvcc process in
parallel, then linked into ``socrates_gb300/libsocgpu.so``.  Objects go to
``socrates_gb300/_build/``.  A build is skipped when the library is newer
than every source.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libsocgpu.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          f"-I{INCLUDE}", f"-I{CSRC}"]
# The generator mirrors the reference's FP64 branch decisions bit for bit:
# no multiply-add contraction there.
PER_FILE = {"cloud_gen.cu": ["-fmad=false"]}

# flux_inst.cu is compiled once per (precision, mode, lanes); see its header.
# The mixed-precision kernels trade IEEE division/square root for the fast
# hardware forms (a few ulp in FP32); their error budget is set by the
# flux/heating-rate tolerances, not by last-bit FP32 rounding.
FLUX_LANES = {0: (16, 32), 1: (8, 16, 32)}


TOOL = PKG / "socgpu_run"
TOOL_MAIN = "run_main.cpp"


def units() -> list[tuple[Path, str, list[str]]]:
    """(source, object stem, extra flags) of every object of the library."""
    out = []
    for src in sorted(list(CSRC.glob("*.cu")) + [p for p in CSRC.glob("*.cpp") if p.name != TOOL_MAIN]):
        if src.name == "flux_inst.cu":
            for prec, lanes_list in FLUX_LANES.items():
                for mode in (0, 1, 2):
                    for lanes in lanes_list:
                        # one object per source (1 solar, 2 infra-red)
                        for src_id, tag in ((2, "ir"), (1, "sw")) if mode else ((2, "ir"),):
                            flags = [f"-DSOCGPU_PREC={prec}", f"-DSOCGPU_MODE={mode}", f"-DSOCGPU_LANES={lanes}",
                                     f"-DSOCGPU_SRC={src_id}"]
                            if prec == 1:
                                flags.append("-use_fast_math")
                            out.append((src, f"flux_{prec}_{mode}_{lanes}_{tag}", flags))
        elif src.name == "flux_phased.cu":
            for prec in (0, 1):
                for mode in (0, 1):
                    flags = [f"-DSOCGPU_PREC={prec}", f"-DSOCGPU_MODE={mode}"]
                    if prec == 1:
                        flags.append("-use_fast_math")
                    out.append((src, f"phased_{prec}_{mode}", flags))
        else:
            out.append((src, src.stem, PER_FILE.get(src.name, [])))
    return out


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsocgpu")


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    if not TOOL.exists():
        return True
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def _compile(unit: tuple[Path, str, list[str]], extra: list[str]) -> Path:
    src, stem, flags = unit
    obj = BUILD / (stem + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *flags, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {stem}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile every CUDA source and link libsocgpu.so; return its path."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    todo = units()
    # the largest objects first, so the slowest compiles start early
    todo.sort(key=lambda u: 0 if u[1].startswith(("flux_", "phased_")) else 1)
    jobs = min(len(todo), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda u: _compile(u, extra or []), todo))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-Xlinker", "-rpath=/usr/local/cuda/lib64",
           *map(str, objs), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # the column-file driver (socgpu_run), linked against the library
    tool_tmp = TOOL.with_suffix(".tmp")
    cmd = [nvcc(), *ARCH, "-std=c++17", "-O2", f"-I{INCLUDE}", f"-I{CSRC}", str(CSRC / TOOL_MAIN),
           str(BUILD / "cdf_io.o"), str(BUILD / "mcica_setup.o"), "-o", str(tool_tmp), f"-L{PKG}", "-lsocgpu", "-cudart", "shared",
           "-Xlinker", "-rpath=$ORIGIN", "-Xlinker", "-rpath=/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of socgpu_run failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tool_tmp, TOOL)
    if verbose:
        print(f"built {LIB} and {TOOL}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
