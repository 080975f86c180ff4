"""GPU tracker (through the C ABI) against the CPU oracle.

FP64 form: per-history traces (element-sequence hash, segment and
collision counts, last element, exit face, end state, final energy and
position) must match bit for bit; element flux tallies, which the GPU sums
with atomics in arbitrary order, must match within 1e-12 relative.
"""
import numpy as np
import pytest

from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import (MC_BC_REFLECT, MC_MODE_EVENT, MC_MODE_HISTORY, MC_SRC_BOX,
                              MC_SRC_MONO, MC_TALLY_SUM, MC_TALLY_SUM_SQ)
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

TALLY_RTOL = 1e-12


def assert_traces_equal(g, o):
    assert g.shape == o.shape
    for f in ("id", "hash", "status", "n_seg", "n_coll", "elem", "face"):
        bad = np.nonzero(g[f] != o[f])[0]
        assert bad.size == 0, f"field {f} differs for {bad.size} histories, first id {g['id'][bad[0]]}"
    for f in ("E", "x", "y", "z"):
        gb = g[f].view(np.uint64)
        ob = o[f].view(np.uint64)
        bad = np.nonzero(gb != ob)[0]
        assert bad.size == 0, f"field {f} not bit-exact for {bad.size} histories"


def assert_tally_close(g, o, rtol=TALLY_RTOL):
    scale = np.maximum(np.abs(o), 1e-300)
    rel = np.abs(g - o) / scale
    nz = o != 0
    assert np.all(g[~nz] == 0)
    assert rel[nz].max() <= rtol, rel[nz].max()


@pytest.fixture(scope="module")
def cube():
    return problems.cube_problem()  # 48,000 tets, 10 nuclides x 10,000 points


@pytest.fixture(scope="module")
def cube_oracle(cube):
    o = Oracle(cube)
    return o.run(100000, seed=1, threads=8)


@pytest.mark.parametrize("mode", [MC_MODE_HISTORY, MC_MODE_EVENT])
def test_cube_fp64_bit_exact(cube, cube_oracle, mode):
    tally_o, tr_o, st_o, _ = cube_oracle
    with Tracker(0) as t:
        t.load(cube)
        st = t.run(100000, seed=1, mode=mode, traces=True)
        tr = t.traces(100000)
        tally = t.tally()
    assert_traces_equal(tr, tr_o)
    assert_tally_close(tally, tally_o)
    assert st.n_seg == st_o["n_seg"] and st.n_coll == st_o["n_coll"]
    assert st.n_leak == st_o["n_leak"] and st.n_absorb == st_o["n_absorb"]
    assert st.n_stuck == 0 and st.n_lost == 0
    assert st.leak_weight == st_o["leak_weight"]


def test_event_small_bank_and_segment_budget(cube, cube_oracle):
    """Refill, re-queue after a segment budget, and the tail kernel."""
    tally_o, tr_o, _, _ = cube_oracle
    with Tracker(0) as t:
        t.load(cube)
        t.run(100000, seed=1, mode=MC_MODE_EVENT, bank_size=3000, max_seg=3, traces=True)
        tr = t.traces(100000)
        tally = t.tally()
    assert_traces_equal(tr, tr_o)
    assert_tally_close(tally, tally_o)


@pytest.mark.parametrize("walk_blocks", [4, 5])
def test_fp64_walk_register_budgets_bit_exact(cube, cube_oracle, walk_blocks):
    """Both builds of the FP64 walk kernel (4 or 5 resident blocks per SM)
    give the oracle's traces; any other value is refused."""
    tally_o, tr_o, _, _ = cube_oracle
    with Tracker(0) as t:
        t.load(cube)
        t.run(100000, seed=1, mode=MC_MODE_EVENT, bank_size=100000, max_seg=64, traces=True, graph=True,
              walk_blocks=walk_blocks)
        assert_traces_equal(t.traces(100000), tr_o)
        assert_tally_close(t.tally(), tally_o)
        with pytest.raises(RuntimeError):
            t.run(1000, seed=1, mode=MC_MODE_EVENT, walk_blocks=3)


def test_lattice_small_fp64_bit_exact():
    p = problems.lattice_problem(nx=3, ny=3, nz=4, height=10.0, n_pts=4000)
    tally_o, tr_o, st_o, _ = Oracle(p).run(20000, first=500, seed=3, threads=8)
    for mode in (MC_MODE_HISTORY, MC_MODE_EVENT):
        with Tracker(0) as t:
            t.load(p)
            t.run(20000, first=500, seed=3, mode=mode, bank_size=4096, traces=True)
            assert_traces_equal(t.traces(20000), tr_o)
            assert_tally_close(t.tally(), tally_o)


def test_reflective_box_source_mono_energy():
    p = problems.cube_problem(n=6, L=6.0, n_nuc=4, n_pts=2000)
    p.bcs = {b: MC_BC_REFLECT for b in range(6)}
    p.source = problems.Source(space=MC_SRC_BOX, energy=MC_SRC_MONO, box_lo=(0.5, 0.5, 0.5),
                               box_hi=(5.5, 5.5, 5.5), mono_E=2.0)
    tally_o, tr_o, st_o, _ = Oracle(p).run(4000, seed=11, threads=8)
    assert st_o["n_leak"] == 0
    for mode in (MC_MODE_HISTORY, MC_MODE_EVENT):
        with Tracker(0) as t:
            t.load(p)
            t.run(4000, seed=11, mode=mode, traces=True)
            assert_traces_equal(t.traces(4000), tr_o)
            assert_tally_close(t.tally(), tally_o)


def test_batches_accumulate_like_openmc_results(cube):
    """SUM / SUM_SQ over batches of batch tally / batch weight."""
    o = Oracle(cube)
    with Tracker(0) as t:
        t.load(cube)
        ref_sum = np.zeros(cube.n_tet)
        ref_sq = np.zeros(cube.n_tet)
        for b in range(3):
            t.run(5000, first=5000 * b, seed=2, accumulate=True)
            tal, _, _, _ = o.run(5000, first=5000 * b, seed=2, threads=8, traces=False)
            ref_sum += tal / 5000
            ref_sq += (tal / 5000) ** 2
        assert t.batches_done() == 3
        assert_tally_close(t.tally(MC_TALLY_SUM), ref_sum, 1e-11)
        assert_tally_close(t.tally(MC_TALLY_SUM_SQ), ref_sq, 1e-11)
        assert np.all(t.tally() == 0)


def test_empty_and_single_history(cube, cube_oracle):
    _, tr_o, _, _ = cube_oracle
    with Tracker(0) as t:
        t.load(cube)
        st = t.run(0, seed=1)
        assert st.n_hist == 0
        for mode in (MC_MODE_HISTORY, MC_MODE_EVENT):
            t.run(1, first=41, seed=1, mode=mode, traces=True)
            assert_traces_equal(t.traces(1), tr_o[41:42])
