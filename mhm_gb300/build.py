"""Build libmhm_gpu.so (CUDA, sm_103a) in-tree, under mhm_gb300/_build/.

Translation units are compiled in parallel with nvcc and linked into one
shared library exposing the C ABI of include/mhm_gpu.h.  FP64 contraction is
disabled on both sides (--fmad=false for device code, -ffp-contract=off for
host code): the kernels evaluate every a*b+c with two roundings, as the
reference's gfortran build does, and fma() only where hmath.h writes it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = BUILD / "libmhm_gpu.so"
# the bounds-checked variant (-DMHM_BOUNDS_CHECK): index tests before every
# data-derived access, failures reported through a device status word
LIB_BC = BUILD / "libmhm_gpu_bc.so"

SOURCES = ["cell_chain.cu", "cell_chain_o6.cu", "cell_chain_o8.cu", "routing.cu", "probes.cu", "mpr.cu", "engine.cu",
           "network.cpp", "netbuild.cpp", "mpr_host.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA extension cannot be built")


def _flags(verbose_ptxas: bool) -> list[str]:
    f = ARCH + [
        "-O3", "-std=c++17", "-lineinfo", "--fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
        "-I", str(CSRC), "-I", str(INCLUDE),
    ]
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    extra = os.environ.get("MHM_NVCC_FLAGS", "").split()
    return f + extra


def _stale(lib: Path = LIB) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + \
        list(CSRC.glob("*.cpp")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose_ptxas: bool = False, quiet: bool = True, bounds_check: bool = False) -> Path:
    """Compile every translation unit for sm_103a and link libmhm_gpu.so
    (with bounds_check: libmhm_gpu_bc.so, objects under _build/bc/)."""
    lib = LIB_BC if bounds_check else LIB
    if not force and not _stale(lib):
        return lib
    odir = BUILD / "bc" if bounds_check else BUILD
    odir.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    flags = _flags(verbose_ptxas) + (["-DMHM_BOUNDS_CHECK"] if bounds_check else [])

    def compile_one(src: str) -> tuple[str, str]:
        obj = odir / (Path(src).stem + ".o")
        cmd = [cc, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        if src.endswith(".cpp"):
            cmd = [cc, "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
                   "-I", str(CSRC), "-I", str(INCLUDE), "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return str(obj), r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if not quiet or verbose_ptxas:
        for _, log in results:
            if log.strip():
                print(log, file=sys.stderr)
    tmp = lib.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *[o for o, _ in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    bc = "--bounds-check" in sys.argv
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, quiet=False, bounds_check=bc))
