"""Builds the in-tree shared library libmacaw_gb300.so for sm_103a.

CUDA translation units go through nvcc with -fmad=false (no contraction of
a*b+c into one rounding, so FP64 results are reproducible against host
arithmetic); host C++ units go through g++ with -ffp-contract=off for the
same reason (aarch64 contracts by default).  Objects are compiled in
parallel and linked into macaw_gb300/libmacaw_gb300.so.
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
LIB = PKG / "libmacaw_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-O3"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]

CU_SOURCES = ["mc_kernels.cu", "mc_api.cu", "mc_noalloc.cu", "mc_serve.cu", "mc_eigen.cu", "mc_persist.cu"]
CXX_SOURCES = ["mc_exodus.cpp", "mc_host.cpp", "mc_gen.cpp", "mc_app.cpp", "mc_tune.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build macaw_gb300")


def _cuda_lib_dir(nvcc: str) -> Path:
    root = Path(nvcc).resolve().parent.parent
    for d in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        if (root / d / "libcudart.so").exists() or (root / d / "libcudart_static.a").exists():
            return root / d
    return root / "lib64"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile (if out of date) and return the path of libmacaw_gb300.so."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "macaw_gb300.h"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    cxx = os.environ.get("CXX", "g++")
    for src in CXX_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append([cxx, *CXX_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
            for fut in [ex.submit(_run, j) for j in jobs]:
                fut.result()
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lpthread",
              "-L" + str(_cuda_lib_dir(nvcc))])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


def ptxas_report() -> str:
    """Register/shared-memory usage of every kernel (nvcc -Xptxas -v)."""
    nvcc = _nvcc()
    out = []
    for src in CU_SOURCES:
        r = subprocess.run([nvcc, *ARCH, *NVCC_FLAGS, "-Xptxas", "-v", "-c", str(CSRC / src), "-o", os.devnull],
                           capture_output=True, text=True)
        out.append(r.stdout + r.stderr)
    return "\n".join(out)


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    if "--ptxas" in sys.argv:
        print(ptxas_report())
