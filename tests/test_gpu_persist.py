"""mc_run_persistent: many batches of two problems in one persistent launch.

The batches (uneven sizes, interleaved between a pin lattice and a cube)
must give, history for history, the FP64 traces of mc_run's event form bit
for bit, and each problem's SUM/SUM_SQ must equal mc_run's over the same
batches within 1e-12 relative -- with one tally slot per batch (no waits)
and with a single slot per problem (each batch waits for the previous one
of its problem to be folded).  A wait limit of one poll must end the run
with MC_ERR_DEVICE and leave the contexts usable.
"""
import numpy as np
import pytest

from macaw_gb300 import MCError, Tracker, problems
from macaw_gb300._lib import (MC_ERR_DEVICE, MC_MODE_EVENT, MC_PREC_FP64, MC_PREC_MIXED, MC_TALLY_SUM,
                              MC_TALLY_SUM_SQ)
from macaw_gb300.tracker import run_persistent

pytestmark = pytest.mark.gpu

# (problem, first history, histories, seed)
PLAN = [("lat", 0, 3000, 5), ("cube", 0, 1000, 6), ("lat", 3000, 500, 5), ("cube", 1000, 4000, 6),
        ("lat", 3500, 2500, 5), ("lat", 6000, 1, 5)]


@pytest.fixture(scope="module")
def probs():
    return {"lat": problems.lattice_problem(nx=5, ny=5, nz=4, height=8.0, n_pts=2000),
            "cube": problems.cube_problem(n=10, L=10.0, n_nuc=5, n_pts=2000)}


def _reference(probs):
    """Each batch through mc_run (event form, accumulate), in plan order."""
    out = {}
    tr = []
    with Tracker(0) as a, Tracker(0) as b:
        ts = {"lat": a, "cube": b}
        for k, t in ts.items():
            t.load(probs[k])
        for k, first, n, seed in PLAN:
            ts[k].run(n, first=first, seed=seed, mode=MC_MODE_EVENT, precision=MC_PREC_FP64, traces=True,
                      accumulate=True)
            tr.append(ts[k].traces(n))
        for k, t in ts.items():
            out[k] = (t.tally(MC_TALLY_SUM), t.tally(MC_TALLY_SUM_SQ), t.batches_done())
    return out, np.concatenate(tr)


@pytest.mark.parametrize("slots", [0, 1])
def test_persistent_equals_event_form(probs, slots):
    ref, ref_tr = _reference(probs)
    with Tracker(0) as a, Tracker(0) as b:
        ts = {"lat": a, "cube": b}
        for k, t in ts.items():
            t.load(probs[k])
            t.run(0)  # tables onto the device
        st, tr = run_persistent([(ts[k], first, n, seed) for k, first, n, seed in PLAN], precision=MC_PREC_FP64,
                                slots=slots, traces=True)
        assert st.n_hist == sum(n for _, _, n, _ in PLAN)
        for f in ("id", "hash", "status", "n_seg", "n_coll", "elem", "face"):
            assert np.array_equal(tr[f], ref_tr[f]), f
        for f in ("E", "x", "y", "z"):
            assert np.array_equal(tr[f].view(np.uint64), ref_tr[f].view(np.uint64)), f
        for k, t in ts.items():
            s, q, nb = ref[k]
            got_s, got_q = t.tally(MC_TALLY_SUM), t.tally(MC_TALLY_SUM_SQ)
            assert t.batches_done() == nb
            for g, r in ((got_s, s), (got_q, q)):
                nz = r != 0
                assert np.all(g[~nz] == 0)
                assert np.all(np.abs(g[nz] - r[nz]) <= 1e-12 * np.abs(r[nz])), k


def test_persistent_mixed_runs_every_history(probs):
    with Tracker(0) as a, Tracker(0) as b:
        ts = {"lat": a, "cube": b}
        for k, t in ts.items():
            t.load(probs[k])
            t.run(0)
        st, _ = run_persistent([(ts[k], first, n, seed) for k, first, n, seed in PLAN], precision=MC_PREC_MIXED,
                               slots=2)
        assert st.n_hist == sum(n for _, _, n, _ in PLAN) and st.n_stuck == 0 and st.n_lost == 0
        mixed = ts["lat"].tally(MC_TALLY_SUM)
    ref, _ = _reference(probs)
    assert abs(mixed.sum() / ref["lat"][0].sum() - 1.0) < 1e-2


def test_bounded_wait_gives_up_and_reports(probs):
    with Tracker(0) as t:
        t.load(probs["lat"])
        t.run(0)
        # one slot: the second batch's histories wait for the first batch's
        # fold, and a limit of one poll cannot cover it
        with pytest.raises(MCError) as ei:
            run_persistent([(t, 0, 20000, 1), (t, 20000, 20000, 1)], slots=1, wait_limit=1)
        assert ei.value.code == MC_ERR_DEVICE
        assert "waited" in str(ei.value)
        # the context still works
        t.reset_tally()
        st = t.run(1000, seed=2)
        assert st.n_hist == 1000
        st, _ = run_persistent([(t, 0, 2000, 1), (t, 2000, 2000, 1)], slots=0)
        assert st.n_hist == 4000
