"""Build recipe for the in-tree CUDA library and the CPU oracle.

The engine is compiled for sm_103a only, without fast math and without FMA contraction
(--fmad=false on the device, -ffp-contract=off on the host side), because the citation choices are
defined bit-for-bit and must match the oracle's arithmetic.  Each translation unit compiles in its
own process; the objects link into paragraph_gb300/_lib/libparagraph_gb300.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libparagraph_gb300.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
    "-I", str(ROOT / "include"),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _compile(src: Path, obj: Path, extra: list[str]) -> str:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
    return r.stderr


def build_library(force: bool = False, verbose_ptxas: bool = False) -> Path:
    srcs = _sources()
    headers = list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    newest = max(p.stat().st_mtime for p in srcs + headers)
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest:
        drv_src = PKG / "abm" / "abm_main.cpp"
        if not DRIVER.exists() or DRIVER.stat().st_mtime < max(drv_src.stat().st_mtime, LIB.stat().st_mtime):
            build_driver()
        return LIB
    objdir = PKG / "_build"
    objdir.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    objs = [objdir / (s.stem + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        logs = list(ex.map(lambda so: _compile(so[0], so[1], extra), zip(srcs, objs)))
    if verbose_ptxas:
        for s, log in zip(srcs, logs):
            print(f"== {s.name}\n{log}")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver()
    return LIB


DRIVER = LIBDIR / "abm"


def build_driver() -> Path:
    """The `abm` command-line driver (C++17), linked against the library with an $ORIGIN rpath."""
    src = PKG / "abm" / "abm_main.cpp"
    cxx = os.environ.get("CXX", "g++")
    tmp = DRIVER.with_suffix(".tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(src), "-L", str(LIBDIR),
           "-lparagraph_gb300", "-Wl,-rpath,$ORIGIN", "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"abm driver build failed:\n{r.stderr}")
    os.replace(tmp, DRIVER)
    return DRIVER


def build_oracle(force: bool = False) -> Path:
    src = ORACLE_DIR / "oracle.c"
    hdr = ORACLE_DIR / "oracle.h"
    newest = max(src.stat().st_mtime, hdr.stat().st_mtime)
    if ORACLE_LIB.exists() and not force and ORACLE_LIB.stat().st_mtime >= newest:
        return ORACLE_LIB
    ORACLE_LIB.parent.mkdir(exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-std=gnu11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", str(src), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, force)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    import sys

    build_library(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv)
    build_oracle(force="--force" in sys.argv)
    print(LIB, ORACLE_LIB)
