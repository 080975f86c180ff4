"""Recorded ray segments (the data of MOOSE's RayTracingExodus output).

The segments of a recorded history chain end to start, start at its source
site and end where its trace ends, number as many as the trace's segments,
and count the sides crossed; the FP64 form's histories are the oracle's, so
the recorded positions close on the oracle's end points bit for bit.
"""
import numpy as np
import pytest

from macaw_gb300 import Tracker, exodus, problems
from macaw_gb300._lib import MC_MODE_EVENT, MC_MODE_HISTORY, MC_PREC_FP64, MC_PREC_MIXED

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cube():
    return problems.cube_problem(n=8, L=8.0, n_nuc=4, n_pts=2000)


@pytest.mark.parametrize("mode,prec", [(MC_MODE_EVENT, MC_PREC_FP64), (MC_MODE_HISTORY, MC_PREC_FP64),
                                       (MC_MODE_EVENT, MC_PREC_MIXED)])
def test_recorded_rays_chain_and_close_on_the_trace(cube, mode, prec, tmp_path):
    n, n_rays, first = 4000, 50, 1000
    with Tracker(0) as t:
        t.load(cube)
        t.enable_rays(n_rays, 100000)
        t.run(n, first=first, seed=4, mode=mode, precision=prec, traces=True, bank_size=1024, max_seg=16)
        seg = t.rays()
        tr = t.traces(n)
        sites = t.sample_sites(n_rays, first=first, seed=4)
    ids = np.unique(seg["id"])
    assert ids.tolist() == list(range(first + 1, first + n_rays + 1))
    for r, pid in enumerate(ids):
        s = seg[seg["id"] == pid]
        assert s.size == tr["n_seg"][r] and np.array_equal(s["segment"], np.arange(s.size))
        assert np.array_equal(s["start"][1:], s["end"][:-1])
        assert s["intersections"][-1] == tr["n_seg"][r] - tr["n_coll"][r]
        end = np.array([tr["x"][r], tr["y"][r], tr["z"][r]])
        if prec == MC_PREC_FP64:
            assert np.array_equal(s["end"][-1], end)
            site = sites[r]
            assert np.array_equal(s["start"][0], [site["x"], site["y"], site["z"]])
        else:
            assert np.allclose(s["end"][-1], end, rtol=0, atol=1e-12)
    if prec == MC_PREC_FP64 and mode == MC_MODE_EVENT:
        _, otr, _, _ = O.Oracle(cube).run(n_rays, first=first, seed=4)
        for r in range(n_rays):
            s = seg[seg["id"] == first + 1 + r]
            assert np.array_equal(s["end"][-1], [otr["x"][r], otr["y"][r], otr["z"][r]])
        exodus.write_rays(str(tmp_path / "r.e"), seg, first_history=first)


def test_rays_off_records_nothing(cube):
    with Tracker(0) as t:
        t.load(cube)
        t.enable_rays(10, 1000)
        t.enable_rays(0, 0)
        t.run(100, seed=4)
        from macaw_gb300._lib import MCError
        with pytest.raises(MCError):
            t.rays()
