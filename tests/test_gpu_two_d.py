"""2-D mode on the GPU against the oracle: FP64 traces bit for bit and
tallies within 1e-12 in the event and history forms; the mixed form keeps
every history in the plane and within 1e-4 of FP64 on a total."""
import numpy as np
import pytest

from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import MC_MODE_EVENT, MC_MODE_HISTORY, MC_PREC_FP64, MC_PREC_MIXED

from oracle import oracle as O

pytestmark = pytest.mark.gpu
N = 20000


@pytest.fixture(scope="module")
def lat2d():
    return problems.lattice_2d_problem(nx=5, ny=5, n_pts=3000)


@pytest.fixture(scope="module")
def ref(lat2d):
    t, tr, st, _ = O.Oracle(lat2d).run(N, seed=8, threads=8)
    return t, tr


@pytest.mark.parametrize("mode", [MC_MODE_EVENT, MC_MODE_HISTORY])
def test_fp64_two_d_matches_the_oracle(lat2d, ref, mode):
    t_ref, tr_ref = ref
    with Tracker(0) as t:
        t.load(lat2d)
        t.run(N, seed=8, mode=mode, precision=MC_PREC_FP64, traces=True, bank_size=4096, max_seg=32)
        got, tr = t.tally(), t.traces(N)
    for f in ("hash", "status", "n_seg", "n_coll", "elem", "face", "E", "x", "y", "z"):
        assert np.array_equal(tr[f], tr_ref[f]), f
    nz = t_ref > 0
    assert np.all(got[~nz] == 0) and np.all(np.abs(got[nz] - t_ref[nz]) <= 1e-12 * t_ref[nz])
    assert np.all(tr["z"] == lat2d.z_2d)


def test_mixed_two_d_stays_in_the_plane(lat2d, ref):
    t_ref, _ = ref
    with Tracker(0) as t:
        t.load(lat2d)
        st = t.run(N, seed=8, precision=MC_PREC_MIXED, traces=True, max_seg=64)
        got, tr = t.tally(), t.traces(N)
    assert st.n_stuck == 0 and st.n_lost == 0
    assert np.all(tr["z"] == lat2d.z_2d)
    assert abs(got.sum() / t_ref.sum() - 1.0) < 1e-4
