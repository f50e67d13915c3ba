"""In-tree build of the engine: libluxum.so (C ABI + sm_103a kernels) and the luxum CLI.

Everything compiles with nvcc/g++ directly (no cmake), translation units in parallel, one
-gencode (sm_103a).  Host code is built with -ffp-contract=off so that the constants and
CPML profiles computed on the host round identically on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libluxum.so"
CLI = PKG / "luxum"
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["lx_kernels.cu", "lx_sweep3d.cu", "lx_api.cu", "lx_yaml.cpp", "lx_hdf5.cpp", "lx_noalloc.cu", "lx_server.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def _deps() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [REPO / "include" / "luxum.h", pathlib.Path(__file__)]


def _stale(out: pathlib.Path, srcs: list[pathlib.Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_library(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """Compiles libluxum.so next to this file; returns its path."""
    BUILD.mkdir(exist_ok=True)
    nv = nvcc()
    common = ["-std=c++17", "-O3", "-DLX_BUILDING_LIBRARY", "-I", str(REPO / "include"),
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden"]
    deps = _deps()
    jobs = []
    objs = []
    for src in LIB_SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + deps):
            cmd = [nv] + common + ["-lineinfo"] + (GENCODE if src.endswith(".cu") else []) + ["-c", str(s), "-o", str(o)]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nv, "-shared", "-o", str(tmp)] + [str(o) for o in objs] + GENCODE + ["-lpthread"], verbose)
        os.replace(tmp, LIB)
    return LIB


def build_cli(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """Compiles the `luxum` command-line driver (links libluxum.so via $ORIGIN)."""
    src = CSRC / "luxum_main.cpp"
    if not src.exists():
        return CLI
    if force or _stale(CLI, [src, LIB] + _deps()):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(REPO / "include"), str(src), "-o", str(CLI),
              "-L", str(PKG), "-lluxum", "-Wl,-rpath,$ORIGIN", "-lpthread"], verbose)
    return CLI


def build(force: bool = False, verbose: bool = False) -> None:
    build_library(force, verbose)
    build_cli(force, verbose)


if __name__ == "__main__":
    import sys

    build(force="--force" in sys.argv, verbose=True)
