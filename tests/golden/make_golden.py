"""Extracts golden vectors from the reference's only gold file.

Source: test/tests/study/gold/openmc_study_rays.e of idaholab/macaw (the
`study_run` Exodiff test, test/tests/study/tests:2-13).  Each EDGE2 element
is one ray segment, its two nodes the segment's start and end; its element
variables hold the ray's aux data after the segment, including the OpenMC
seeds stored as doubles (src/raykernels/CollisionKernel.C:157-159,
src/userobjects/OpenMCStudy.C:345-347).

Writes, next to this script:
  openmc_study_rays_seeds.npz   per segment the ray id, the intersection
                                index, the energy, the aux particle id and
                                the three seed doubles;
  openmc_study_rays_points.npz  per segment the ray id, the intersection
                                index, the energy, the tracking seed and the
                                start and end coordinates.

Usage (the reference checkout is required; nothing is assumed about where
it lives):
    python tests/golden/make_golden.py PATH_TO_MACAW_CHECKOUT
or with the environment variable MACAW_REFERENCE set to that path.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np


def main(argv: list[str]) -> int:
    ref = argv[1] if len(argv) > 1 else os.environ.get("MACAW_REFERENCE")
    if not ref:
        print(__doc__, file=sys.stderr)
        return 2
    gold = Path(ref) / "test/tests/study/gold/openmc_study_rays.e"
    from scipy.io import netcdf_file

    f = netcdf_file(str(gold), "r", mmap=False)
    names = [b"".join(r).decode().strip("\x00") for r in f.variables["name_elem_var"][:]]
    V = {n: np.array(f.variables[f"vals_elem_var{i + 1}eb1"][0]) for i, n in enumerate(names)}
    xyz = np.stack([np.array(f.variables[k][:], np.float64) for k in ("coordx", "coordy", "coordz")], axis=1)
    conn = np.array(f.variables["connect1"][:], np.int64) - 1
    here = Path(__file__).resolve().parent
    np.savez_compressed(
        here / "openmc_study_rays_seeds.npz",
        ray_id=V["ray_id"].astype(np.int64),
        intersections=V["intersections"].astype(np.int64),
        energy=V["aux_energy"],
        aux_id=V["aux_id"].astype(np.int64),
        seed_tracking=V["aux_seed_tracking"],
        seed_source=V["aux_seed_source"],
        seed_urr=V["aux_seed_URR"],
    )
    np.savez_compressed(
        here / "openmc_study_rays_points.npz",
        ray_id=V["ray_id"].astype(np.int64),
        intersections=V["intersections"].astype(np.int64),
        energy=V["aux_energy"],
        seed_tracking=V["aux_seed_tracking"],
        start=xyz[conn[:, 0]],
        end=xyz[conn[:, 1]],
    )
    print(f"wrote {here}/openmc_study_rays_{{seeds,points}}.npz ({conn.shape[0]} segments)", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
