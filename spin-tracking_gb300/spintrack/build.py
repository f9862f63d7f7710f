"""In-tree build of the CUDA engine (libspintrack.so) and the spintrack CLI.

Everything is compiled for sm_103a only (GB300), translation units in
parallel, outputs under spin-tracking_gb300/_build/.  No cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # spin-tracking_gb300/
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
INCLUDE = REPO_ROOT / "include"
BUILD = PKG_ROOT / "_build"
LIB = BUILD / "libspintrack.so"
CLI = BUILD / "spintrack"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code keeps the reference's rounding: no contraction of a * b + c into an FMA
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              f"-I{INCLUDE}", f"-I{CSRC}"]
UNITS = ["st_kernels.cu", "st_kernels_ext.cu", "st_api.cpp", "st_noalloc.cu", "st_adjoint.cu", "st_ensemble.cu",
         "st_spectrum.cu"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the spintrack engine needs the CUDA toolkit")
    return cand


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> Path:
    """Compile libspintrack.so and the CLI; returns the library path."""
    nvcc = _nvcc()
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "spintrack.h"]
    objs = []
    jobs = []
    for u in UNITS:
        src = CSRC / u
        obj = BUILD / (u + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            extra = ["-Xptxas", "-v"] if (ptxas_info and u.endswith(".cu")) else []
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(lambda c: _run(c, verbose or ptxas_info), jobs))
    if force or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"], verbose)
    cli_src = CSRC / "st_cli.cpp"
    if force or _stale(CLI, [cli_src, LIB]):
        _run([nvcc, "-O2", "-std=c++17", f"-I{INCLUDE}", str(cli_src), "-o", str(CLI),
              f"-L{BUILD}", "-lspintrack", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"], verbose)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
