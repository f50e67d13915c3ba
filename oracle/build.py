"""Build recipe of the oracle (test infrastructure): liboracle.so from luxum_oracle.c.

gcc -O3 -fopenmp -ffp-contract=off: -O3 as the reference's own build (src/solvers/CMakeLists.txt:22);
OpenMP mirrors the reference's `omp parallel for` loops (used when the CPU baseline is timed);
no FMA contraction and no fast-math, so results are the same at any optimisation level and on
x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liboracle.so"
SRC = HERE / "luxum_oracle.c"
HDR = HERE.parent / "include" / "luxum.h"


def build_oracle(force: bool = False) -> pathlib.Path:
    OUT_DIR.mkdir(exist_ok=True)
    if not force and LIB.exists() and LIB.stat().st_mtime > max(SRC.stat().st_mtime, HDR.stat().st_mtime,
                                                                 pathlib.Path(__file__).stat().st_mtime):
        return LIB
    cc = shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-std=c11", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
