"""mc_run_noalloc: the batch run for callers that cannot allocate device memory.

Those callers (an application whose memory pool owns the GPU, a serving
process with a fixed HBM budget) get the event-form tracker with its scratch
in a fixed array inside the library; they pass their own device buffers for
the results.  These tests call the entry point through the C ABI:

* twice in a row, in the FP64 and the mixed form, with a bank of 8,192 and
  with the maximum (bank_size 0), each result against mc_run on the same
  histories with the same bank and tail hand-over: FP64 traces bit for bit
  and tallies within the 1e-12 relative tolerance of the parity tests;
  mixed traces bit for bit too (same kernels, same visits) and tallies
  within the same 1e-12;
* in a fresh process, the device's free memory before and after the first
  call must be equal (the array and kernels were loaded by mc_ctx_create);
* with a bank above the maximum, or fields it cannot honour, it must refuse.

They must pass alone in a fresh process and after the other tests.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import MC_MODE_EVENT, MC_PREC_FP64, MC_PREC_MIXED, TRACE_DTYPE, RunDesc, lib

pytestmark = pytest.mark.gpu

N = 30000
RTOL = 1e-12
TAIL = 2048  # same tail hand-over in both entry points, so the mixed visits match


def _desc(first, n, bank, traces, precision=MC_PREC_FP64, tail=TAIL):
    return RunDesc(first, n, bank, 7, precision, MC_MODE_EVENT, 0, 0, int(traces), 0, 0, 0, 0, 0, 0, tail, None,
                   None)


@pytest.mark.parametrize("precision,bank", [(MC_PREC_FP64, 8192), (MC_PREC_FP64, 0), (MC_PREC_MIXED, 8192),
                                            (MC_PREC_MIXED, 0)])
def test_noalloc_matches_mc_run_twice_in_a_row(precision, bank):
    torch = pytest.importorskip("torch")
    p = problems.cube_problem(n=12, L=12.0, n_nuc=6, n_pts=3000)
    ref_bank = bank if bank > 0 else 16384  # bank_size 0 is the maximum here
    with Tracker(0) as t:
        t.load(p)
        t.run(0)  # puts mesh, tables and source on the device
        h = t._h
        for call, first in enumerate((0, 5000)):
            t.reset_tally()
            t.run(N, first=first, seed=7, mode=MC_MODE_EVENT, precision=precision, bank_size=ref_bank, traces=True,
                  tail=TAIL)
            ref_tally = t.tally()
            ref_tr = t.traces(N)
            ref_st = t.stats()

            tally = torch.zeros(p.n_tet, dtype=torch.float64, device="cuda")
            trace_buf = torch.zeros(N * TRACE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
            torch.cuda.synchronize()
            d = _desc(first, N, bank, True, precision)
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
            assert st.n_stuck == 0 and st.n_lost == 0
            if precision == MC_PREC_FP64:
                assert st.leak_weight == ref_st.leak_weight


_FRESH = r"""
import ctypes as C, sys
import torch
sys.path.insert(0, sys.argv[1])
from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import MC_MODE_EVENT, MC_PREC_FP64, MC_PREC_MIXED, RunDesc, lib
p = problems.cube_problem(n=8, L=8.0, n_nuc=4, n_pts=2000)
with Tracker(0) as t:
    t.load(p)
    t.run(0)
    tally = torch.zeros(p.n_tet, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    out = []
    for prec in (MC_PREC_FP64, MC_PREC_MIXED):
        d = RunDesc(0, 20000, 0, 3, prec, MC_MODE_EVENT, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, None, None)
        free0 = torch.cuda.mem_get_info()[0]
        rc = lib.mc_run_noalloc(t._h, C.byref(d), C.c_void_p(tally.data_ptr()), None)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        assert rc == 0, lib.mc_last_error(t._h).decode()
        out.append(f"{free0} {free1}")
print(" ".join(out))
"""


def test_first_noalloc_call_of_a_fresh_process_takes_no_device_memory():
    pytest.importorskip("torch")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FRESH, root], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    v = [int(x) for x in r.stdout.split()[-4:]]
    assert v[0] == v[1], f"FP64 first call: free device memory {v[0]} -> {v[1]}"
    assert v[2] == v[3], f"mixed first call: free device memory {v[2]} -> {v[3]}"


def test_noalloc_rejects_a_bank_above_the_maximum_and_unsupported_fields():
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
        for field, value, msg in (("n_batches", 2, b"pipelined"), ("sort_queue", 9, b"ordering"),
                                  ("graph", 1, b"graph")):
            d = _desc(0, 100, 1024, False)
            setattr(d, field, value)
            rc = lib.mc_run_noalloc(t._h, C.byref(d), C.c_void_p(tally.data_ptr()), None)
            assert rc != 0 and msg in lib.mc_last_error(t._h), field
        t.enable_rays(4, 16)
        d = _desc(0, 100, 1024, False)
        rc = lib.mc_run_noalloc(t._h, C.byref(d), C.c_void_p(tally.data_ptr()), None)
        assert rc != 0 and b"ray recording" in lib.mc_last_error(t._h)
