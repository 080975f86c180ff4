"""Tally definitions on the GPU against the oracle.

Each definition (estimator, scores, energy filter; OpenMCTally,
src/userobjects/OpenMCTally.C:30-101) must give, in the FP64 form, the
oracle's tally within 1e-12 relative (atomic summation order) with
per-history traces bit for bit, in the event and history forms, through
pipelined batches and through the serving path.  The mixed form must count
collisions exactly with the collision estimator's total score.
"""
import numpy as np
import pytest

from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import (MC_EST_COLLISION, MC_EST_TRACKLENGTH, MC_MODE_EVENT, MC_MODE_HISTORY,
                              MC_PREC_FP64, MC_PREC_MIXED, MC_SCORE_ABSORPTION, MC_SCORE_FLUX, MC_SCORE_SCATTER,
                              MC_SCORE_TOTAL, MC_SRC_MONO, MC_SRC_POINT, MC_TALLY_SUM)
from macaw_gb300.serve import Job, Server

from oracle import oracle as O

pytestmark = pytest.mark.gpu

EDGES = np.array([1.0e-5, 1.0, 1.0e3, 1.0e5, 1.0e6, 2.0e7])
DEFS = {
    "tl_flux_total_binned": problems.TallyDef(MC_EST_TRACKLENGTH, (MC_SCORE_FLUX, MC_SCORE_TOTAL), EDGES),
    "coll_all_binned": problems.TallyDef(MC_EST_COLLISION, (MC_SCORE_FLUX, MC_SCORE_TOTAL, MC_SCORE_SCATTER,
                                                            MC_SCORE_ABSORPTION), EDGES),
    "coll_flux": problems.TallyDef(MC_EST_COLLISION, (MC_SCORE_FLUX,), None),
}
N = 20000


def close(a, b, rtol=1e-12):
    nz = b != 0
    return np.all(a[~nz] == 0) and np.all(np.abs(a[nz] - b[nz]) <= rtol * np.abs(b[nz]))


@pytest.fixture(scope="module")
def lattice():
    # dense enough that histories collide: 15 cm tall 5x5 lattice, small grids
    return problems.lattice_problem(nx=5, ny=5, nz=6, height=15.0, n_pts=3000)


@pytest.fixture(scope="module")
def oracle_results(lattice):
    out = {}
    for k, d in DEFS.items():
        lattice.tally = d
        o = O.Oracle(lattice)
        t, tr, st, _ = o.run(N, seed=3, threads=8)
        out[k] = (t, tr, st)
    lattice.tally = None
    return out


@pytest.mark.parametrize("key", list(DEFS))
@pytest.mark.parametrize("mode", [MC_MODE_EVENT, MC_MODE_HISTORY])
def test_fp64_tally_definitions_match_the_oracle(lattice, oracle_results, key, mode):
    ref, tr_ref, st_ref = oracle_results[key]
    with Tracker(0) as t:
        t.load(lattice)
        t.configure_tally(DEFS[key])
        assert t.tally_size() == ref.size
        st = t.run(N, seed=3, mode=mode, precision=MC_PREC_FP64, traces=True, bank_size=4096, max_seg=32)
        got = t.tally()
        tr = t.traces(N)
    for f in ("hash", "status", "n_seg", "n_coll", "elem", "face"):
        assert np.array_equal(tr[f], tr_ref[f]), f
    assert close(got, ref), key
    if DEFS[key].estimator == MC_EST_COLLISION and MC_SCORE_TOTAL in DEFS[key].scores:
        j = DEFS[key].scores.index(MC_SCORE_TOTAL)
        assert got.reshape(-1, len(DEFS[key].scores))[:, j].sum() == st.n_coll == st_ref["n_coll"]


def test_mixed_collision_total_counts_collisions(lattice):
    d = DEFS["coll_all_binned"]
    with Tracker(0) as t:
        t.load(lattice)
        t.configure_tally(d)
        st = t.run(N, seed=3, precision=MC_PREC_MIXED, max_seg=64)
        got = t.tally().reshape(-1, 4)
    assert st.n_stuck == 0 and st.n_lost == 0
    assert got[:, 1].sum() == st.n_coll
    nz = got[:, 1] > 0
    assert np.allclose(got[nz, 2] + got[nz, 3], got[nz, 1], rtol=1e-12)


def test_pipelined_batches_with_a_tally_definition(lattice):
    d = DEFS["tl_flux_total_binned"]
    sizes = [3000, 1000, 4000, 2000]
    with Tracker(0) as t:
        t.load(lattice)
        t.configure_tally(d)
        first = 0
        for s in sizes:
            t.run(s, first=first, seed=3, accumulate=True)
            first += s
        ref = t.tally(MC_TALLY_SUM)
        t.reset_tally()
        t.run(sum(sizes), seed=3, accumulate=True, batch_sizes=sizes, bank_size=2048)
        assert close(t.tally(MC_TALLY_SUM), ref)
        assert t.batches_done() == len(sizes)


def test_serving_uses_the_tally_definition(lattice):
    d = DEFS["coll_all_binned"]
    lattice.tally = d
    try:
        srv = Server([lattice], precision=MC_PREC_FP64, bank=4096, max_slots=2)
        job = Job(0, 5000, 21, (3.1, 3.2, 7.5), 1.0e6)
        k = srv.submit(job)
        while not srv.idle():
            srv.step()
        got = srv.result(k)
        srv.close()
        with Tracker(0) as t:
            t.load(lattice)
            t.set_source(problems.Source(space=MC_SRC_POINT, energy=MC_SRC_MONO, point=job.point,
                                         mono_E=job.energy))
            t.run(job.n_histories, seed=job.seed, precision=MC_PREC_FP64)
            ref = t.tally()
    finally:
        lattice.tally = None
    assert got.size == ref.size == lattice.n_tet * (len(EDGES) - 1) * 4
    assert ref.sum() > 0 and close(got, ref)


def test_bad_tally_definitions_are_rejected(lattice):
    from macaw_gb300._lib import MCError
    with Tracker(0) as t:
        t.load(lattice)
        with pytest.raises(MCError):
            t.configure_tally(problems.TallyDef(MC_EST_TRACKLENGTH, (MC_SCORE_SCATTER,), None))
        with pytest.raises(MCError):
            t.configure_tally(problems.TallyDef(MC_EST_COLLISION, (MC_SCORE_FLUX,), np.array([1.0, 0.5])))
        with pytest.raises(MCError):
            t.configure_tally(problems.TallyDef(7, (MC_SCORE_FLUX,), None))
        assert t.tally_size() == lattice.n_tet
