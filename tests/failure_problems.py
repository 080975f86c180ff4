"""Small problems that drive the tracker into its failure paths.

Each failure is made on the host side of the data (a table, a source, a
limit); none of them makes a GPU fault, trap or hang.  The reference's
error conventions these stand for: OpenMC's fatal_error on bad data at
setup (src/userobjects/OpenMCStudy.C:130-131), a ray that cannot be
claimed by any element (OpenMCStudy.C:290-294), and a particle OpenMC
kills inside the collision kernel (src/raykernels/CollisionKernel.C:187-189).
"""
from __future__ import annotations

import numpy as np

from macaw_gb300 import problems
from macaw_gb300._lib import MC_BC_REFLECT, MC_BC_VACUUM, MC_SRC_MONO, MC_SRC_POINT, MC_SRC_WATT
from macaw_gb300.problems import Material, Nuclide, Problem, Source


def _cube(nuc: Nuclide, src: Source, bc: int, n: int = 4, L: float = 4.0, density: float = 0.05) -> Problem:
    xyz, tv, blk, bid = problems.cube_mesh(n, L)
    mat = Material(1, np.array([0], np.int32), np.array([density]))
    return Problem("failure_cube", xyz, tv, blk, bid, [nuc], [mat], np.array([0], np.int32),
                   np.array([1], np.int32), src, {b: bc for b in range(6)}, hash_bins=64)


def grid(n: int = 200) -> np.ndarray:
    return np.geomspace(problems.E_MIN, problems.E_MAX, n)


def zero_range_problem() -> Problem:
    """A table that uploads (every value finite, 0 <= sigma_s <= sigma_t)
    but has sigma_t = 0 between 0.3 and 3 MeV, where a Watt source puts a
    large share of its neutrons: those histories end with a bad cross
    section at their first segment."""
    E = grid()
    st = 5.0 / np.sqrt(E) + 2.0
    st[(E > 3e5) & (E < 3e6)] = 0.0
    nuc = Nuclide(E, st, 0.5 * st, 12.0)
    return _cube(nuc, Source(space=MC_SRC_POINT, energy=MC_SRC_WATT, point=(2.0, 2.0, 2.0)), MC_BC_VACUUM)


def outside_source_problem() -> Problem:
    """A point source outside the mesh: no history can be located."""
    E = grid()
    st = 5.0 / np.sqrt(E) + 2.0
    nuc = Nuclide(E, st, 0.5 * st, 12.0)
    return _cube(nuc, Source(space=MC_SRC_POINT, energy=MC_SRC_MONO, mono_E=1e6, point=(10.0, 2.0, 2.0)),
                 MC_BC_VACUUM)


def pure_scatterer_problem() -> Problem:
    """A reflective cube of a heavy pure scatterer (no absorption, target
    mass ratio 200): a history loses about 1% of its energy per collision
    and cannot leak, so it walks for thousands of collisions; a low segment
    limit ends every history as stuck."""
    E = grid()
    st = np.full(E.size, 2.0)
    nuc = Nuclide(E, st, st.copy(), 200.0)
    return _cube(nuc, Source(space=MC_SRC_POINT, energy=MC_SRC_MONO, mono_E=1e6, point=(2.0, 2.0, 2.0)),
                 MC_BC_REFLECT, density=0.5)


BAD_TABLES = [
    ("nan sigma_t", lambda E: (np.where(E > 1e3, np.nan, 1.0), np.full(E.size, 0.5), 1.0)),
    ("inf sigma_t", lambda E: (np.where(E > 1e3, np.inf, 1.0), np.full(E.size, 0.5), 1.0)),
    ("inf sigma_s", lambda E: (np.full(E.size, 1.0), np.where(E > 1e3, np.inf, 0.5), 1.0)),
    ("negative sigma_s", lambda E: (np.full(E.size, 1.0), np.where(E > 1e3, -0.5, 0.5), 1.0)),
    ("sigma_s above sigma_t", lambda E: (np.full(E.size, 1.0), np.full(E.size, 1.5), 1.0)),
    ("inf awr", lambda E: (np.full(E.size, 1.0), np.full(E.size, 0.5), np.inf)),
]
