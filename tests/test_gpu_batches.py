"""Batches of uneven size run through one event pipeline.

Batch b scores into tally slot b mod 8 (up to eight batches in flight) and
is folded into SUM/SUM_SQ, normalised by its size, when its last particle
ends; the next batches' births fill the bank meanwhile.  The result must equal one mc_run
per batch: SUM and SUM_SQ within 1e-12, per-history traces bit for bit.
"""
import numpy as np
import pytest

from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import (MC_MODE_EVENT, MC_MODE_HISTORY, MC_PREC_FP64, MC_PREC_MIXED, MC_TALLY_SUM,
                              MC_TALLY_SUM_SQ)

pytestmark = pytest.mark.gpu

SIZES = [3000, 5000, 1000, 7000, 2500]
# more batches than tally slots: slots are reused once their batch drained
SIZES_LONG = [900, 1500, 400, 2200, 700, 1300, 300, 1800, 1000, 600, 2500, 800]


def close(a, b, rtol=1e-12):
    nz = b != 0
    return np.all(a[~nz] == 0) and np.all(np.abs(a[nz] - b[nz]) <= rtol * np.abs(b[nz]))


@pytest.fixture(scope="module")
def cube():
    return problems.cube_problem(n=10, L=10.0, n_nuc=5, n_pts=3000)


def _separate(cube, sizes):
    with Tracker(0) as t:
        t.load(cube)
        first = 0
        trs = []
        for s in sizes:
            t.run(s, first=first, seed=5, mode=MC_MODE_EVENT, accumulate=True, traces=True)
            trs.append(t.traces(s))
            first += s
        return t.tally(MC_TALLY_SUM), t.tally(MC_TALLY_SUM_SQ), np.concatenate(trs)


@pytest.fixture(scope="module")
def separate(cube):
    return _separate(cube, SIZES)


@pytest.mark.parametrize("bank", [1024, 6000])
def test_more_batches_than_tally_slots(cube, bank):
    s_ref, sq_ref, tr_ref = _separate(cube, SIZES_LONG)
    n = sum(SIZES_LONG)
    with Tracker(0) as t:
        t.load(cube)
        st = t.run(n, seed=5, bank_size=bank, accumulate=True, traces=True, batch_sizes=SIZES_LONG)
        assert st.n_hist == n and t.batches_done() == len(SIZES_LONG)
        tr = t.traces(n)
        for f in ("hash", "status", "n_seg", "n_coll", "elem", "face"):
            assert np.array_equal(tr[f], tr_ref[f]), f
        assert close(t.tally(MC_TALLY_SUM), s_ref)
        assert close(t.tally(MC_TALLY_SUM_SQ), sq_ref)
        assert np.all(t.tally() == 0)


@pytest.mark.parametrize("mode,bank", [(MC_MODE_EVENT, 2048), (MC_MODE_EVENT, 40000), (MC_MODE_HISTORY, 0)])
def test_pipelined_batches_equal_separate_runs(cube, separate, mode, bank):
    s_ref, sq_ref, tr_ref = separate
    n = sum(SIZES)
    with Tracker(0) as t:
        t.load(cube)
        st = t.run(n, seed=5, mode=mode, bank_size=bank, accumulate=True, traces=True, batch_sizes=SIZES)
        assert st.n_hist == n
        assert t.batches_done() == len(SIZES)
        tr = t.traces(n)
        for f in ("hash", "status", "n_seg", "n_coll", "elem", "face"):
            assert np.array_equal(tr[f], tr_ref[f]), f
        assert close(t.tally(MC_TALLY_SUM), s_ref)
        assert close(t.tally(MC_TALLY_SUM_SQ), sq_ref)
        assert np.all(t.tally() == 0)


def test_graph_replayed_event_cycles_are_bit_exact(cube, separate):
    s_ref, sq_ref, tr_ref = separate
    n = sum(SIZES)
    with Tracker(0) as t:
        t.load(cube)
        t.run(n, seed=5, mode=MC_MODE_EVENT, bank_size=3000, max_seg=8, sort_queue=5, graph=True,
              accumulate=True, traces=True, batch_sizes=SIZES)
        tr = t.traces(n)
        for f in ("hash", "status", "n_seg", "n_coll", "elem", "face"):
            assert np.array_equal(tr[f], tr_ref[f]), f
        assert close(t.tally(MC_TALLY_SUM), s_ref)


def test_autotune_returns_usable_parameters(cube):
    with Tracker(0) as t:
        t.load(cube)
        t.run(3000, seed=9, accumulate=True)
        s0, q0, b0 = t.tally(MC_TALLY_SUM), t.tally(MC_TALLY_SUM_SQ), t.batches_done()
        for prec in (MC_PREC_FP64, MC_PREC_MIXED):
            params, rate = t.autotune(trial=20000, bank_size=8192, precision=prec)
            assert rate > 0
        # the pipelined trials leave the accumulators and the batch count as they were
        assert np.array_equal(t.tally(MC_TALLY_SUM), s0) and np.array_equal(t.tally(MC_TALLY_SUM_SQ), q0)
        assert t.batches_done() == b0 and np.all(t.tally() == 0)
        st = t.run(5000, seed=5, accumulate=True, **params)
        assert st.n_hist == 5000 and st.n_stuck == 0


def test_pipelined_mixed_batches_keep_every_particle(cube):
    n = sum(SIZES)
    with Tracker(0) as t:
        t.load(cube)
        st = t.run(n, seed=5, mode=MC_MODE_EVENT, precision=MC_PREC_MIXED, bank_size=4096,
                   max_seg=64, accumulate=True, batch_sizes=SIZES)
        assert st.n_hist == n and st.n_stuck == 0 and st.n_lost == 0
        assert t.batches_done() == len(SIZES)


def test_batch_arguments_are_checked(cube):
    from macaw_gb300 import MCError
    with Tracker(0) as t:
        t.load(cube)
        with pytest.raises(MCError, match="add up"):
            t.run(100, accumulate=True, batch_sizes=[40, 50])
        with pytest.raises(MCError, match="accumulate"):
            t.run(90, accumulate=False, batch_sizes=[40, 50])


def test_batch_results_stream_each_batch_sum(cube):
    """batch_results: buffer b holds SUM once batch b is folded in, equal to
    the SUM after b+1 separate runs; host sites feed the pipelined batches."""
    sizes = SIZES_LONG
    with Tracker(0) as t:
        t.load(cube)
        sites = t.sample_sites(sum(sizes), seed=5)
        ref = []
        first = 0
        for s in sizes:
            t.run(s, first=first, seed=5, accumulate=True, sites=sites[first:first + s])
            ref.append(t.tally(MC_TALLY_SUM).copy())
            first += s
        t.reset_tally()
        outs = [np.zeros(t.tally_size()) for _ in sizes]
        t.run(sum(sizes), seed=5, accumulate=True, bank_size=2048, batch_sizes=sizes, sites=sites,
              batch_results=outs)
        assert t.batches_done() == len(sizes)
        # batches are folded in birth order, each as soon as it and every
        # older batch have drained
        for b in range(len(sizes)):
            assert close(outs[b], ref[b]), b
        with pytest.raises(Exception):
            t.run(sum(sizes), seed=5, accumulate=False, batch_sizes=sizes, batch_results=outs)


def test_host_sites_reach_every_pipelined_batch(cube):
    """Host sites of later batches are copied while the first batches walk;
    births wait for their copy: every history equals the one born from the
    device-sampled site (same site, same stream), bit for bit."""
    sizes = SIZES_LONG * 2
    n = sum(sizes)
    with Tracker(0) as t:
        t.load(cube)
        t.run(n, seed=7, bank_size=1024, accumulate=True, traces=True, batch_sizes=sizes)
        tr_dev = t.traces(n).copy()
        sites = t.sample_sites(n, seed=7)
        t.reset_tally()
        t.run(n, seed=7, bank_size=1024, accumulate=True, traces=True, batch_sizes=sizes, sites=sites)
        tr_host = t.traces(n)
        assert t.batches_done() == len(sizes)
    for f in ("hash", "status", "n_seg", "n_coll", "elem", "face"):
        assert np.array_equal(tr_host[f], tr_dev[f]), f
    assert np.array_equal(tr_host["E"].view(np.uint64), tr_dev["E"].view(np.uint64))
