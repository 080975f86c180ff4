"""The GPU walk and ReflectRayBC against the reference's gold rays.

The same runs as tests/test_gold_walk.py (449 straight collision-free runs
of the gold file's rays, started as host source sites on the 5 x 5 x 1
reflective study box cut into tets, transparent materials): the library's
recorded segments, through the C ABI, must cross the same 919 hex faces and
wall reflection points as MOOSE's trace to 1e-12 of the box half-width,
and equal the oracle's recorded segments bit for bit in FP64 (every
segment's start, end, element, energy and tracking state) in the event and
history forms.  The mixed form (float walk, FP64 re-solve near edges) must
cross them within 1e-4 cm (1e-5 of the box width; a float direction
reflected at a grazing angle moves its crossings by about 1e-5 cm).
"""
import numpy as np
import pytest

import gold_walk as G
from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import MC_MODE_EVENT, MC_MODE_HISTORY, MC_PREC_MIXED, SITE_DTYPE
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12 * 5.0
MIXED_TOL = 1e-4  # cm
SEG_LIMIT = 200


@pytest.fixture(scope="module")
def runs(golden_dir):
    return G.gold_runs(dict(np.load(golden_dir / "openmc_study_rays_points.npz")))


@pytest.fixture(scope="module")
def sites(runs):
    s = G.sites(runs)
    out = np.zeros(len(runs), SITE_DTYPE)
    for j, k in enumerate(("x", "y", "z", "u", "v", "w", "E", "wgt")):
        out[k] = s[:, j]
    return out


@pytest.fixture(scope="module")
def oracle_rays(runs, sites):
    o = Oracle(problems.study_box_problem())
    o.set_segment_limit(SEG_LIMIT)
    o.enable_rays(len(runs), SEG_LIMIT)
    _, tr, _, _ = o.run(len(runs), sites=sites)
    return o.rays(), tr


@pytest.mark.parametrize("mode", [MC_MODE_EVENT, MC_MODE_HISTORY])
def test_gpu_walk_matches_gold_and_oracle(runs, sites, oracle_rays, mode):
    rays_o, tr_o = oracle_rays
    with Tracker(0) as t:
        t.load(problems.study_box_problem())
        t.set_segment_limit(SEG_LIMIT)
        t.enable_rays(len(runs), SEG_LIMIT)
        st = t.run(len(runs), sites=sites, mode=mode, traces=True)
        rays = t.rays()
        tr = t.traces(len(runs))
    assert st.n_coll == 0 and st.n_stuck == len(runs) and st.n_lost == 0
    n, worst = G.compare(runs, rays)
    assert n == 919 and worst <= TOL, f"largest crossing difference {worst:.3e} cm"
    # bit for bit against the oracle
    assert rays.size == rays_o.size == len(runs) * SEG_LIMIT
    for f in ("id", "segment", "intersections", "elem", "seed_tracking"):
        assert np.array_equal(rays[f], rays_o[f]), f
    for f in ("start", "end", "E", "wgt"):
        assert np.array_equal(rays[f].view(np.uint64), rays_o[f].view(np.uint64)), f
    for f in ("hash", "status", "n_seg", "elem"):
        assert np.array_equal(tr[f], tr_o[f]), f


def test_gpu_mixed_walk_crosses_the_gold_faces(runs, sites):
    with Tracker(0) as t:
        t.load(problems.study_box_problem())
        t.set_segment_limit(SEG_LIMIT)
        t.enable_rays(len(runs), SEG_LIMIT)
        st = t.run(len(runs), sites=sites, precision=MC_PREC_MIXED)
        rays = t.rays()
    assert st.n_coll == 0 and st.n_lost == 0
    n_pts = 0
    for i, run in enumerate(runs):
        seg = rays[rays["id"] == i + 1]
        seg = seg[np.argsort(seg["segment"])]
        # float crossing points lie within MIXED_TOL of a face: loosen the filter accordingly
        ends = [p for p in seg["end"] if np.min(np.abs(p[0] - G.HEX_XY)) <= MIXED_TOL or
                np.min(np.abs(p[1] - G.HEX_XY)) <= MIXED_TOL or np.min(np.abs(p[2] - G.HEX_Z)) <= MIXED_TOL]
        got = []
        for p in ends:
            if not got or np.max(np.abs(p - got[-1])) > MIXED_TOL:
                got.append(p)
        want = run["points"]
        assert len(got) >= want.shape[0]
        err = np.max(np.abs(np.array(got[:want.shape[0]]) - want))
        assert err <= MIXED_TOL, f"run {i}: {err:.2e} cm"
        n_pts += want.shape[0]
    assert n_pts == 919
