"""History sharding through the library, on one GPU.

What each rank of a multi-GPU run does (macaw_gb300/shard.py): track its
own contiguous range of history indices with mc_run (first_history), then
sum the FP64 tallies.  Here the two ranks' ranges run one after the other
on the one GPU; their traces must equal a single call's bit for bit and
their summed tally must equal its tally within 1e-12 relative."""
import numpy as np
import pytest

from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import MC_MODE_EVENT, MC_MODE_HISTORY, MC_PREC_FP64
from macaw_gb300.shard import history_range

pytestmark = pytest.mark.gpu

N = 20001


@pytest.mark.parametrize("mode", [MC_MODE_EVENT, MC_MODE_HISTORY])
def test_two_ranges_sum_to_one_call(mode):
    p = problems.lattice_problem(nx=5, ny=5, nz=4, height=8.0, n_pts=2000)
    with Tracker(0) as t:
        t.load(p)
        t.run(N, seed=11, mode=mode, precision=MC_PREC_FP64, traces=True)
        whole_t, whole_tr = t.tally(), t.traces(N)
        parts_t, parts_tr = np.zeros_like(whole_t), []
        for rank in range(2):
            first, n = history_range(N, rank, 2)
            t.reset_tally()
            t.run(n, first=first, seed=11, mode=mode, precision=MC_PREC_FP64, traces=True)
            parts_t += t.tally()
            parts_tr.append(t.traces(n))
    tr = np.concatenate(parts_tr)
    for f in ("id", "hash", "status", "n_seg", "n_coll", "elem", "face"):
        assert np.array_equal(tr[f], whole_tr[f]), f
    nz = whole_t != 0
    assert np.array_equal(nz, parts_t != 0)
    assert np.all(np.abs(parts_t[nz] - whole_t[nz]) <= 1e-12 * whole_t[nz])
