"""2-D mode (CollisionKernel z_coord) on the oracle.

In a 2-D problem MaCaw zeroes the z component of every source and scattered
direction (OpenMCStudy.C:355-356, CollisionKernel.C:200-202) and keeps
collision points at z = z_coord (:177-179).  Histories therefore stay in the
plane, and the infinite-medium balances of 3-D transport still hold for the
planar flights: mean track length 1/Sigma_a, mean collisions 1/(1-c).
"""
import numpy as np
import pytest

from macaw_gb300 import problems
from macaw_gb300._lib import MC_BC_REFLECT, MC_SRC_BOX, MC_SRC_MONO

from oracle import oracle as O


def test_histories_stay_in_the_plane():
    p = problems.lattice_2d_problem(nx=3, ny=3, n_pts=500)
    t, tr, st, _ = O.Oracle(p).run(2000, seed=2, threads=4)
    assert st["n_stuck"] == 0 and st["n_lost"] == 0
    assert np.all(tr["z"] == p.z_2d)
    # more segments per history than 3-D in the same cells would not prove much; the
    # tally is nonzero only where histories went and sums to the total track length
    assert t.sum() > 0


def _flat(sig_t=0.5, c=0.6):
    p = problems.lattice_2d_problem(nx=2, ny=2, n_pts=50)
    E = np.geomspace(1e-5, 2e7, 50)
    p.nuclides = [problems.Nuclide(E, np.full(50, sig_t), np.full(50, c * sig_t), 5000.0)]
    p.materials = [problems.Material(m, np.array([0], np.int32), np.array([1.0])) for m in (1, 2, 3)]
    p.bcs = {b: MC_BC_REFLECT for b in range(6)}
    p.source = problems.Source(space=MC_SRC_BOX, energy=MC_SRC_MONO, box_lo=(0.1, 0.1, 0.0), box_hi=(2.4, 2.4, 1.0),
                               mono_E=1.0e6)
    return p


def test_planar_infinite_medium_balances():
    sig_t, c = 0.5, 0.6
    p = _flat(sig_t, c)
    n = 4000
    t, tr, st, _ = O.Oracle(p).run(n, seed=3, threads=4)
    assert st["n_leak"] == 0 and st["n_absorb"] == n
    mean_l = t.sum() / n
    assert abs(mean_l * sig_t * (1 - c) - 1.0) < 0.05
    assert abs(st["n_coll"] / n * (1 - c) - 1.0) < 0.05
    assert np.all(tr["z"] == p.z_2d)


def test_two_d_differs_from_three_d():
    p = problems.lattice_2d_problem(nx=3, ny=3, n_pts=500)
    t2, tr2, _, _ = O.Oracle(p).run(500, seed=2)
    p.z_2d = None
    t3, tr3, _, _ = O.Oracle(p).run(500, seed=2)
    assert not np.array_equal(tr2["hash"], tr3["hash"])
