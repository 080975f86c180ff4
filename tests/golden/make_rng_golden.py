"""Extracts the RNG golden vectors from the reference's only gold file.

Source: test/tests/study/gold/openmc_study_rays.e (MaCaw's `study_run`
Exodiff test, test/tests/study/tests:2-13).  Each EDGE2 element is one ray
segment; its element variables hold the ray's aux data after the segment,
including the OpenMC seeds stored as doubles (src/raykernels/
CollisionKernel.C:157-159, src/userobjects/OpenMCStudy.C:345-347).

Written to openmc_study_rays_seeds.npz: per segment the ray id, the
intersection index, the energy and the three seed doubles, plus the aux
particle id.  Run in a checkout that has the reference at REF (default
/root/reference):  python tests/golden/make_rng_golden.py
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np


def main() -> None:
    ref = Path(os.environ.get("REF", "/root/reference"))
    gold = ref / "test/tests/study/gold/openmc_study_rays.e"
    from scipy.io import netcdf_file

    f = netcdf_file(str(gold), "r", mmap=False)
    names = [b"".join(r).decode().strip("\x00") for r in f.variables["name_elem_var"][:]]
    V = {n: np.array(f.variables[f"vals_elem_var{i + 1}eb1"][0]) for i, n in enumerate(names)}
    out = Path(__file__).resolve().parent / "openmc_study_rays_seeds.npz"
    np.savez_compressed(
        out,
        ray_id=V["ray_id"].astype(np.int64),
        intersections=V["intersections"].astype(np.int64),
        energy=V["aux_energy"],
        aux_id=V["aux_id"].astype(np.int64),
        seed_tracking=V["aux_seed_tracking"],
        seed_source=V["aux_seed_source"],
        seed_urr=V["aux_seed_URR"],
    )
    print(f"wrote {out} ({V['ray_id'].size} segments)", file=sys.stderr)


if __name__ == "__main__":
    main()
