"""Builds the oracle (test infrastructure only) into oracle/_build/.

The reference itself (MOOSE + OpenMC + libMesh + MPI + HDF5) cannot be
built here, so there is no oracle/_ref; the oracle is the C restatement in
mc_oracle.c, compiled with -ffp-contract=off so its double arithmetic is
one IEEE operation per source operation on every host architecture.

The same library also carries a build of the synthetic problem generators
(macaw_gb300/csrc/mc_gen.cpp, host code) so that a CPU-only run of the
oracle -- bench.py's reference arm -- can build its inputs without loading
the CUDA tracker library.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "libmc_oracle.so"
GEN = HERE.parent / "macaw_gb300" / "csrc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    src = HERE / "mc_oracle.c"
    deps = [src, HERE / "mc_oracle.h", GEN / "mc_gen.cpp", GEN / "mc_core.cuh",
            HERE.parent / "include" / "macaw_gb300.h"]
    if force or not LIB.exists() or max(d.stat().st_mtime for d in deps) > LIB.stat().st_mtime:
        cc = os.environ.get("CC", "gcc")
        cxx = os.environ.get("CXX", "g++")
        o1, o2 = OUT / "mc_oracle.o", OUT / "mc_gen.o"
        _run([cc, "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-std=c11", "-c", str(src), "-o", str(o1)])
        _run([cxx, "-O2", "-ffp-contract=off", "-fPIC", "-std=c++17", "-c", str(GEN / "mc_gen.cpp"), "-o", str(o2)])
        tmp = LIB.with_suffix(".so.tmp")
        _run([cxx, "-shared", "-fopenmp", str(o1), str(o2), "-o", str(tmp), "-lm"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
