"""Build recipe for the native library ``libnetsci_gb300.so``.

CUDA translation units go through nvcc for sm_103a only; host-only C++
units through g++. Objects are compiled in parallel and relinked only when
a source or header changed. No cmake; the same recipe runs on x86-64 and
aarch64 hosts.
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
BUILD = ROOT / "_build" / "netsci_gb300"
LIB = PKG / "libnetsci_gb300.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["ksg_d1.cu", "ksg_d2.cu", "ksg_d3.cu", "ksg.cu", "ksg_tie.cu", "ksg_noalloc.cu", "apsp.cu",
              "rowstats.cu", "node_com.cu", "ksg_grid.cu", "ksg_grid_rec.cu", "ceiling.cu"]
CPP_SOURCES = ["cuarray.cpp", "npy.cpp", "engine.cpp", "ksg_cpu.cpp", "netcalc.cpp", "serve.cpp", "capi.cpp",
               "dcd.cpp", "netchem.cpp"]


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.rglob("*.h")))


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: str) -> Path:
    path = CSRC / src
    obj = BUILD / (src + ".o")
    if not _stale(obj, [path] + _headers() + [Path(__file__)]):
        return obj
    inc = ["-I", str(INCLUDE), "-I", str(CSRC)]
    if src.endswith(".cu"):
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xptxas", "-warn-spills", *inc, "-c", str(path), "-o", str(obj)]
    else:
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function", *inc,
               "-I", str(CUDA_HOME / "include"), "-c", str(path), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    """Compile and link the library in-tree; returns its path."""
    if not Path(NVCC).exists() and shutil.which("nvcc") is None:
        raise RuntimeError("nvcc not found; set CUDA_HOME")
    BUILD.mkdir(parents=True, exist_ok=True)
    sources = CU_SOURCES + CPP_SOURCES
    workers = min(len(sources), max(2, os.cpu_count() or 2))
    with ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(_compile, sources))
    if _stale(LIB, objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
