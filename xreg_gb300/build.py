"""Builds libxreg_gb300.so in-tree (xreg_gb300/_build/) with nvcc for sm_103a.

The translation units compile in parallel; the shared library links the CUDA
runtime statically so it loads without any library-path set-up.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
LIB_PATH = BUILD_DIR / "libxreg_gb300.so"
SOURCES = ["xr_capi.cu", "xr_geom.cu", "xr_raycast.cu", "xr_metrics.cu", "xr_noalloc.cu", "xr_preproc.cu", "xr_probe.cu",
           "xr_cmaes.cpp", "xr_dfo.cpp", "xr_regi.cpp", "xr_io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
    "-I" + str(REPO_DIR / "include"), "-I" + str(CSRC),
]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libxreg_gb300")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(exist_ok=True)
    headers = [*sorted((REPO_DIR / "include").glob("*.h")), *sorted(CSRC.glob("*.h")), *sorted(CSRC.glob("*.cuh"))]
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD_DIR / (Path(src).stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers, Path(__file__)]):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({r.returncode}):\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB_PATH, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB_PATH), *map(str, objs)]
        run(cmd)
    return LIB_PATH


if __name__ == "__main__":
    p = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(p)
