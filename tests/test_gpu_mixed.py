"""Mixed-precision form against the FP64 form (which is bit-exact to the oracle).

Same histories, same random-number streams: the element flux tallies of
the two forms must agree to a mean relative difference of 1e-4 over the
scored elements (the precision target), the total track length to 1e-5, and
no particle may be lost or stuck.
"""
import numpy as np
import pytest

from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import MC_MODE_EVENT, MC_MODE_HISTORY, MC_PREC_FP64, MC_PREC_MIXED

pytestmark = pytest.mark.gpu


def rel_diff(a, b):
    nz = b > 0
    return np.abs(a[nz] - b[nz]) / b[nz]


@pytest.fixture(scope="module")
def lattice():
    return problems.lattice_problem(nx=5, ny=5, nz=6, height=15.0, n_pts=4000)


@pytest.fixture(scope="module")
def fp64_tally(lattice):
    with Tracker(0) as t:
        t.load(lattice)
        t.run(200000, seed=9, mode=MC_MODE_EVENT, precision=MC_PREC_FP64)
        return t.tally()


@pytest.mark.parametrize("mode,walk", [(MC_MODE_EVENT, {}), (MC_MODE_EVENT, {"refill": True, "max_seg": 64}),
                                       (MC_MODE_EVENT, {"sort_queue": 9, "max_seg": 96, "graph": True}),
                                       (MC_MODE_HISTORY, {})])
def test_mixed_matches_fp64_tallies(lattice, fp64_tally, mode, walk):
    with Tracker(0) as t:
        t.load(lattice)
        st = t.run(200000, seed=9, mode=mode, precision=MC_PREC_MIXED, **walk)
        m = t.tally()
    assert st.n_hist == 200000
    assert st.n_stuck == 0 and st.n_lost == 0 and st.n_badxs == 0
    assert st.n_fallback < 0.05 * st.n_seg
    r = rel_diff(m, fp64_tally)
    print(f"mixed mode={mode}: mean rel {r.mean():.3e} max {r.max():.3e} fallback "
          f"{st.n_fallback / st.n_seg:.3e}")
    assert r.mean() <= 1e-4
    assert abs(m.sum() - fp64_tally.sum()) <= 1e-5 * fp64_tally.sum()


def test_mixed_reflective_box_keeps_every_particle():
    """All-reflective box: a leak would show as a lost weight, a walk that
    loses its element as stuck/lost; neither may happen."""
    from macaw_gb300._lib import MC_BC_REFLECT, MC_SRC_BOX, MC_SRC_MONO
    p = problems.cube_problem(n=6, L=6.0, n_nuc=4, n_pts=2000)
    p.bcs = {b: MC_BC_REFLECT for b in range(6)}
    p.source = problems.Source(space=MC_SRC_BOX, energy=MC_SRC_MONO, box_lo=(0.1, 0.1, 0.1),
                               box_hi=(5.9, 5.9, 5.9), mono_E=2.0)
    with Tracker(0) as t:
        t.load(p)
        st = t.run(20000, seed=4, mode=MC_MODE_EVENT, precision=MC_PREC_MIXED)
    assert st.n_leak == 0 and st.n_stuck == 0 and st.n_lost == 0
    assert st.n_absorb + st.n_cutoff == 20000
