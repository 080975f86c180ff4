"""Tally definitions on the oracle: estimators, scores, energy filter.

OpenMCTally (src/userobjects/OpenMCTally.C:30-101) takes an estimator, a
list of scores and filters (cell, universe, energy).  The element tally is
laid out [element][energy bin][score].  These checks use identities that
hold exactly or up to summation order:
  - energy bins that cover the whole table range add up to the unfiltered
    track-length flux;
  - the collision estimator's total score counts collisions (weight 1);
  - its scatter and absorption scores add up to its total;
  - with constant cross sections, total = Sigma_t * flux per segment;
and one statistical one: collision and track-length flux estimate the same
flux in an infinite (reflective) medium.
"""
import numpy as np
import pytest

from macaw_gb300 import problems
from macaw_gb300._lib import (MC_BC_REFLECT, MC_EST_COLLISION, MC_EST_TRACKLENGTH, MC_SCORE_ABSORPTION,
                              MC_SCORE_FLUX, MC_SCORE_SCATTER, MC_SCORE_TOTAL, MC_SRC_BOX, MC_SRC_MONO)

from oracle import oracle as O

EDGES = np.array([1.0e-5, 1.0, 1.0e3, 1.0e5, 1.0e6, 2.0e7])


@pytest.fixture(scope="module")
def cube():
    return problems.cube_problem(n=6, L=12.0, n_nuc=4, n_pts=2000)


def _run(p, tally, n=3000, seed=5):
    p.tally = tally
    o = O.Oracle(p)
    t, tr, st, _ = o.run(n, seed=seed, threads=4)
    p.tally = None
    return t, tr, st


def test_energy_bins_add_up_to_the_unfiltered_flux(cube):
    flat, tr0, _ = _run(cube, None)
    binned, tr1, _ = _run(cube, problems.TallyDef(MC_EST_TRACKLENGTH, (MC_SCORE_FLUX,), EDGES))
    assert np.array_equal(tr0, tr1)  # the tally definition does not change the histories
    b = binned.reshape(cube.n_tet, len(EDGES) - 1, 1).sum(axis=(1, 2))
    nz = flat > 0
    assert np.all(b[~nz] == 0)
    assert np.allclose(b[nz], flat[nz], rtol=1e-12, atol=0)
    # more than one bin actually scores
    assert np.count_nonzero(binned.reshape(cube.n_tet, -1).sum(axis=0)) >= 3


def test_energy_filter_drops_energies_outside_the_edges(cube):
    flat, _, _ = _run(cube, None)
    part, _, _ = _run(cube, problems.TallyDef(MC_EST_TRACKLENGTH, (MC_SCORE_FLUX,), np.array([1.0e5, 2.0e7])))
    assert 0 < part.sum() < flat.sum()


def test_collision_total_counts_collisions_and_partial_scores_add_up(cube):
    sc = (MC_SCORE_FLUX, MC_SCORE_TOTAL, MC_SCORE_SCATTER, MC_SCORE_ABSORPTION)
    t, _, st = _run(cube, problems.TallyDef(MC_EST_COLLISION, sc, None))
    t = t.reshape(cube.n_tet, 1, 4)
    assert t[:, 0, 1].sum() == st["n_coll"]
    tot = t[:, 0, 1]
    nz = tot > 0
    assert np.allclose(t[nz, 0, 2] + t[nz, 0, 3], tot[nz], rtol=1e-12)
    assert np.all(t[:, 0, 2] >= 0) and np.all(t[:, 0, 3] >= 0)


def _flat_box(sig_t=0.4, c=0.7):
    p = problems.cube_problem(n=4, L=8.0, n_nuc=1, n_pts=50)
    E = np.geomspace(1e-5, 2e7, 50)
    p.nuclides = [problems.Nuclide(E, np.full(50, sig_t), np.full(50, c * sig_t), 200.0)]
    p.materials = [problems.Material(1, np.array([0], np.int32), np.array([1.0]))]
    p.bcs = {b: MC_BC_REFLECT for b in range(6)}
    p.source = problems.Source(space=MC_SRC_BOX, energy=MC_SRC_MONO, box_lo=(0, 0, 0), box_hi=(8, 8, 8),
                               mono_E=1.0e6)
    return p


def test_track_length_total_is_sigma_t_times_flux():
    p = _flat_box()
    t, _, _ = _run(p, problems.TallyDef(MC_EST_TRACKLENGTH, (MC_SCORE_FLUX, MC_SCORE_TOTAL), None), n=2000)
    t = t.reshape(p.n_tet, 2)
    assert np.allclose(t[:, 1], 0.4 * t[:, 0], rtol=1e-12)


def test_collision_and_track_length_flux_agree_in_an_infinite_medium():
    p = _flat_box()
    tl, _, _ = _run(p, None, n=4000)
    co, _, st = _run(p, problems.TallyDef(MC_EST_COLLISION, (MC_SCORE_FLUX,), None), n=4000)
    # total flux per source particle is 1/Sigma_a for both estimators
    assert st["n_coll"] > 10000
    assert abs(co.sum() / tl.sum() - 1.0) < 0.03
