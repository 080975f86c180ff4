"""Failure paths of the oracle, made on the host (tests/failure_problems.py):
bad tables are refused at upload; a zero total cross section ends a
history as bad-xs; a source outside the mesh loses every history; the
segment limit ends runaway histories as stuck.  The GPU library's side is
tests/test_gpu_failures.py."""
import numpy as np
import pytest

import failure_problems as F
from macaw_gb300 import problems
from oracle.oracle import Oracle


@pytest.mark.parametrize("name,make", F.BAD_TABLES)
def test_oracle_refuses_bad_tables(name, make):
    E = F.grid()
    st, ss, awr = make(E)
    o = Oracle()
    with pytest.raises(RuntimeError):
        o._ck(o_add(o, E, st, ss, awr), name)


def o_add(o, E, st, ss, awr):
    from oracle.oracle import _p, lib
    E, st, ss = (np.ascontiguousarray(a, np.float64) for a in (E, st, ss))
    return lib.oracle_add_nuclide(o.h, E.size, _p(E), _p(st), _p(ss), awr)


def test_zero_total_cross_section_ends_histories_as_bad_xs():
    _, tr, st, _ = Oracle(F.zero_range_problem()).run(2000, seed=3)
    bad = tr["status"] == 6
    assert st["n_badxs"] == bad.sum() > 100
    # born in the zero range (no segment walked), or scattered into it later
    assert (tr["n_seg"][bad] == 0).sum() > 100
    assert st["n_hist"] == 2000 and st["n_stuck"] == 0 and st["n_lost"] == 0


def test_source_outside_the_mesh_loses_every_history():
    _, tr, st, _ = Oracle(F.outside_source_problem()).run(500, seed=3)
    assert st["n_lost"] == 500 and np.all(tr["status"] == 5) and st["n_seg"] == 0


def test_segment_limit_ends_runaway_histories():
    o = Oracle(F.pure_scatterer_problem())
    o.set_segment_limit(1000)
    _, tr, st, _ = o.run(300, seed=3)
    assert st["n_stuck"] == 300 and np.all(tr["status"] == 4) and np.all(tr["n_seg"] == 1000)
    assert st["n_coll"] > 300 * 100


def test_default_segment_limit_follows_the_mesh_size():
    o = Oracle(F.pure_scatterer_problem())  # 384 tets
    assert o.segment_limit() == 65536
    o = Oracle(problems.cube_problem(n=20, n_nuc=1, n_pts=100))  # 48,000 tets: cbrt -> 37
    assert o.segment_limit() == 4096 * 37
    o.set_segment_limit(123)
    assert o.segment_limit() == 123
