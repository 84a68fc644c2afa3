"""Builds the in-tree native libraries.

  libmahyco_gb300.so  - the product: host runtime (C++) + sm_103a CUDA kernels,
                        exporting the C ABI of include/hydro_gb300.h
  mahyco_gb300_run    - drop-in command-line driver (deck in, VTK out;
                        tools_src/: driver.cc + the asynchronous VTK writer)

Kernels are compiled for sm_103a only, with --fmad=false and IEEE division /
square root so that FP64 results are bit-identical to the reference's
x86-64 build (which has no fused multiply-add).  Host C++ is compiled with
-ffp-contract=off for the same reason (GCC fuses a*b+c by default on
aarch64).

Usage: python -m mahyco_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libmahyco_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true",
    "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC",
    "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
             "-fno-fast-math", "-Wall"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build "
                       "mahyco_gb300")


def _sources():
    cu = sorted((CSRC / "kernels").glob("*.cu")) + sorted((CSRC / "host").glob("*.cu"))
    cc = sorted((CSRC / "host").glob("*.cc"))
    return cu, cc


def _includes():
    return ["-I", str(ROOT / "include"), "-I", str(CSRC)]


def _compile(cmd: list[str], log: Path) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    log.write_text(" ".join(cmd) + "\n" + res.stdout + res.stderr)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stderr}")


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    cu, cc = _sources()
    headers = (list(CSRC.rglob("*.h")) + list(CSRC.rglob("*.cuh")) +
               [ROOT / "include" / "hydro_gb300.h"])
    jobs = []
    objs = []
    for src in cu:
        obj = OUT / (src.stem + ".cu.o")
        objs.append(obj)
        if force or _newer(obj, [src, *headers]):
            jobs.append(([nvcc, *ARCH, *NVCC_FLAGS, *_includes(), "-c", str(src),
                          "-o", str(obj)], OUT / (src.stem + ".cu.log")))
    for src in cc:
        obj = OUT / (src.stem + ".cc.o")
        objs.append(obj)
        if force or _newer(obj, [src, *headers]):
            jobs.append(([os.environ.get("CXX", "g++"), *CXX_FLAGS, *_includes(),
                          "-I", "/usr/local/cuda/include", "-c", str(src), "-o",
                          str(obj)], OUT / (src.stem + ".cc.log")))
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        list(ex.map(lambda j: _compile(*j), jobs))
    if force or jobs or not LIB.exists():
        _compile([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs),
                  "-lcudart"], OUT / "link.log")
    tools = PKG / "tools_src"
    drv_srcs = sorted(tools.glob("*.cc"))
    if drv_srcs:
        drv = OUT / "mahyco_gb300_run"
        if force or _newer(drv, [*drv_srcs, *tools.glob("*.h"), LIB]):
            _compile([os.environ.get("CXX", "g++"), *CXX_FLAGS, "-pthread", *_includes(),
                      "-I", str(tools), *map(str, drv_srcs), "-o", str(drv), "-L", str(OUT),
                      "-lmahyco_gb300", f"-Wl,-rpath,{OUT}"], OUT / "driver.log")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
