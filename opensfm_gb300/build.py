"""Builds the native parts of the package in-tree.

* ``opensfm_gb300/libgbba.so`` -- the CUDA kernels for sm_103a, the C++ host
  layer and the C ABI declared in ``include/gbba.h``.
* ``oracle/_build/liboracle.so`` -- the FP64 CPU oracle (test
  infrastructure, built here so the tests and the bench's CPU-baseline leg
  can load it; the product never links it).

Translation units compile in parallel; nothing is rebuilt when the object is
newer than its sources.
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
BUILD = PKG / "_build"
LIB = PKG / "libgbba.so"
ORACLE = ROOT / "oracle"
ORACLE_BUILD = ORACLE / "_build"
ORACLE_LIB = ORACLE_BUILD / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"] + ARCH


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build opensfm_gb300")


def _headers(directory: Path) -> list[Path]:
    return sorted(list(directory.glob("*.h")) + list(directory.glob("*.cuh")) + list(directory.glob("*.inc")) +
                  [ROOT / "include" / "gbba.h"])


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    if "spill" in proc.stderr and "0 bytes spill" not in proc.stderr:
        sys.stderr.write(proc.stderr)


def build_library(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    sources = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    hdrs = _headers(CSRC)
    jobs = []
    objs = []
    for src in sources:
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append([nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    ORACLE_BUILD.mkdir(exist_ok=True)
    sources = sorted(ORACLE.glob("*.cpp"))
    deps = sources + sorted(ORACLE.glob("*.h"))
    if _stale(ORACLE_LIB, deps):
        cxx = os.environ.get("CXX", "g++")
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", *map(str, sources), "-o", str(tmp)])
        os.replace(tmp, ORACLE_LIB)
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(2) as ex:
        a = ex.submit(build_library, verbose)
        b = ex.submit(build_oracle, verbose)
        a.result()
        b.result()


if __name__ == "__main__":
    build_all(verbose=True)
