"""mc_run_noalloc: the batch run for callers that cannot allocate device memory.

Those callers (an application whose memory pool owns the GPU, a serving
process with a fixed HBM budget) get the event-form tracker with its scratch
in a fixed array inside the library; they pass their own device buffers for
the results.  This test calls the entry point through the C ABI twice in a
row and checks each result against mc_run on the same histories: traces
bit for bit, tallies within the 1e-12 relative tolerance of the parity
tests.  It must pass alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import MC_MODE_EVENT, MC_PREC_FP64, TRACE_DTYPE, RunDesc, lib

pytestmark = pytest.mark.gpu

N = 30000
RTOL = 1e-12


def _desc(first, n, bank, traces):
    return RunDesc(first, n, bank, 7, MC_PREC_FP64, MC_MODE_EVENT, 0, 0, int(traces), 0, 0, 0, 0, 0, 0, 0, None, None)


def test_noalloc_matches_mc_run_twice_in_a_row():
    torch = pytest.importorskip("torch")
    p = problems.cube_problem(n=12, L=12.0, n_nuc=6, n_pts=3000)
    with Tracker(0) as t:
        t.load(p)
        t.run(0)  # puts mesh, tables and source on the device
        h = t._h
        for call, first in enumerate((0, 5000)):
            t.reset_tally()
            t.run(N, first=first, seed=7, mode=MC_MODE_EVENT, bank_size=8192, traces=True)
            ref_tally = t.tally()
            ref_tr = t.traces(N)
            ref_st = t.stats()

            tally = torch.zeros(p.n_tet, dtype=torch.float64, device="cuda")
            trace_buf = torch.zeros(N * TRACE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
            torch.cuda.synchronize()
            d = _desc(first, N, 8192, True)
            rc = lib.mc_run_noalloc(h, C.byref(d), C.c_void_p(tally.data_ptr()), C.c_void_p(trace_buf.data_ptr()))
            assert rc == 0, lib.mc_last_error(h).decode()
            torch.cuda.synchronize()
            got_tally = tally.cpu().numpy()
            got_tr = trace_buf.cpu().numpy().view(TRACE_DTYPE)
            st = t.stats()

            for f in ("id", "hash", "status", "n_seg", "n_coll", "elem", "face"):
                assert np.array_equal(got_tr[f], ref_tr[f]), f"call {call}: trace field {f} differs"
            assert np.array_equal(got_tr["E"].view(np.uint64), ref_tr["E"].view(np.uint64))
            nz = ref_tally != 0
            assert np.all(got_tally[~nz] == 0)
            assert np.all(np.abs(got_tally[nz] - ref_tally[nz]) <= RTOL * ref_tally[nz]), f"call {call}"
            assert st.n_hist == N and st.n_seg == ref_st.n_seg and st.n_coll == ref_st.n_coll
            assert st.leak_weight == ref_st.leak_weight


def test_noalloc_rejects_a_bank_above_the_maximum():
    torch = pytest.importorskip("torch")
    p = problems.cube_problem(n=4, L=4.0, n_nuc=2, n_pts=500)
    with Tracker(0) as t:
        t.load(p)
        t.run(0)
        tally = torch.zeros(p.n_tet, dtype=torch.float64, device="cuda")
        d = _desc(0, 100, 16384 + 1, False)
        rc = lib.mc_run_noalloc(t._h, C.byref(d), C.c_void_p(tally.data_ptr()), None)
        assert rc != 0
        assert b"exceeds the no-allocation maximum" in lib.mc_last_error(t._h)
