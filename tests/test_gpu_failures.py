"""Failure paths of the GPU library, made on the host (no GPU fault, trap or
hang is involved): the same problems as tests/test_failures.py through the
C ABI.  Bad tables are refused by mc_nuclide_add with MC_ERR_ARG; a zero
total cross section, a source outside the mesh and the segment limit end
histories with a status the host reads (bad-xs, lost, stuck) while the run
itself returns 0, with traces bit for bit equal to the oracle's."""
import numpy as np
import pytest

import failure_problems as F
from macaw_gb300 import MCError, Tracker, problems
from macaw_gb300._lib import MC_ERR_ARG, MC_MODE_EVENT, MC_MODE_HISTORY
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,make", F.BAD_TABLES)
def test_library_refuses_bad_tables(name, make):
    E = F.grid()
    st, ss, awr = make(E)
    with Tracker(0) as t:
        with pytest.raises(MCError) as ei:
            t.add_nuclide(E, st, ss, awr)
        assert ei.value.code == MC_ERR_ARG, name


def _same(tr, tr_o):
    for f in ("hash", "status", "n_seg", "n_coll", "elem", "face"):
        assert np.array_equal(tr[f], tr_o[f]), f
    assert np.array_equal(tr["E"].view(np.uint64), tr_o["E"].view(np.uint64))


@pytest.mark.parametrize("mode", [MC_MODE_EVENT, MC_MODE_HISTORY])
def test_zero_total_cross_section_ends_histories_as_bad_xs(mode):
    p = F.zero_range_problem()
    _, tr_o, st_o, _ = Oracle(p).run(2000, seed=3)
    with Tracker(0) as t:
        t.load(p)
        st = t.run(2000, seed=3, mode=mode, traces=True)
        tr = t.traces(2000)
    assert st.n_badxs == st_o["n_badxs"] > 100
    _same(tr, tr_o)


def test_source_outside_the_mesh_loses_every_history():
    p = F.outside_source_problem()
    with Tracker(0) as t:
        t.load(p)
        st = t.run(500, seed=3, traces=True)
        tr = t.traces(500)
    assert st.n_lost == 500 and st.n_hist == 500 and np.all(tr["status"] == 5)


@pytest.mark.parametrize("mode", [MC_MODE_EVENT, MC_MODE_HISTORY])
def test_segment_limit_ends_runaway_histories(mode):
    p = F.pure_scatterer_problem()
    o = Oracle(p)
    o.set_segment_limit(1000)
    _, tr_o, _, _ = o.run(300, seed=3)
    with Tracker(0) as t:
        t.load(p)
        assert t.segment_limit() == 65536  # the default for 384 tets
        t.set_segment_limit(1000)
        assert t.segment_limit() == 1000
        st = t.run(300, seed=3, mode=mode, traces=True)
        tr = t.traces(300)
    assert st.n_stuck == 300 and np.all(tr["n_seg"] == 1000)
    _same(tr, tr_o)


def test_default_segment_limit_follows_the_mesh_size():
    with Tracker(0) as t:
        t.load(problems.cube_problem(n=20, n_nuc=1, n_pts=100))
        assert t.segment_limit() == 4096 * 37 == Oracle(problems.cube_problem(n=20, n_nuc=1, n_pts=100)).segment_limit()
