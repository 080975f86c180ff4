"""Builds the oracle (test infrastructure only) into oracle/_build/.

The reference itself (MOOSE + OpenMC + libMesh + MPI + HDF5) cannot be
built here, so there is no oracle/_ref; the oracle is the C restatement in
mc_oracle.c, compiled with -ffp-contract=off so its double arithmetic is
one IEEE operation per source operation on every host architecture.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "libmc_oracle.so"


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    src = HERE / "mc_oracle.c"
    hdr = HERE / "mc_oracle.h"
    if force or not LIB.exists() or max(src.stat().st_mtime, hdr.stat().st_mtime) > LIB.stat().st_mtime:
        cc = os.environ.get("CC", "gcc")
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [cc, "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=c11",
               str(src), "-o", str(tmp), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
