"""The oracle's tet walk and reflections against the reference's gold rays.

Between two collisions a ray of the reference's gold file is pure geometry
(tests/gold_walk.py): the 919 collision-free segments of rays 60-89 give 449
straight runs whose 919 end points are hex-face crossings and wall
reflections of MOOSE's trace on the 5 x 5 x 1 reflective box of
test/tests/study/openmc_study.i.  Started at the midpoint of each run's first
segment, in the run's direction, on the same box cut into Kuhn tets, with
transparent materials, the oracle's walk must cross the same hex faces and
reflect at the same points, to 1e-12 of the box half-width (5 cm).
"""
import numpy as np
import pytest

import gold_walk as G
from macaw_gb300 import problems
from oracle.oracle import Oracle

TOL = 1e-12 * 5.0  # absolute, cm: 1e-12 of the box half-width
SEG_LIMIT = 200    # the longest run crosses 14 hex faces; a hex crossing takes at most a few tet segments


@pytest.fixture(scope="module")
def gold(golden_dir):
    return dict(np.load(golden_dir / "openmc_study_rays_points.npz"))


@pytest.fixture(scope="module")
def runs(gold):
    return G.gold_runs(gold)


def test_gold_polylines_chain(gold):
    # each segment starts where the previous one of its ray ended
    rid, inter = gold["ray_id"], gold["intersections"]
    for r in np.unique(rid):
        idx = np.where(rid == r)[0]
        idx = idx[np.argsort(inter[idx])]
        assert np.array_equal(inter[idx], np.arange(idx.size))
        assert np.array_equal(gold["start"][idx[1:]], gold["end"][idx[:-1]])


def test_runs_are_the_collision_free_segments(gold, runs):
    # 919 segments keep their energy and draw one tracking number; every
    # end point of theirs lies on a hex face or a wall
    assert sum(len(r["segments"]) for r in runs) == 919
    assert len(runs) == 449
    for r in runs:
        for p in r["points"]:
            assert G.on_hex_face(p)


def test_box_mesh_matches_the_study_input():
    p = problems.study_box_problem()
    assert p.n_tet == 5 * 5 * 1 * 6
    assert np.array_equal(p.xyz.min(axis=0), [-5.0, -5.0, -5.0])
    assert np.array_equal(p.xyz.max(axis=0), [5.0, 5.0, 5.0])
    assert np.bincount(p.tet_block).tolist() == [144, 6]  # the centre hex in block 1
    assert set(np.unique(p.tet_side_bid)) == {-1, 0, 1, 2, 3, 4, 5}


def test_oracle_walk_matches_gold_crossings_and_reflections(runs):
    o = Oracle(problems.study_box_problem())
    o.set_segment_limit(SEG_LIMIT)
    o.enable_rays(len(runs), SEG_LIMIT)
    _, tr, st, _ = o.run(len(runs), sites=G.sites(runs))
    # nothing collides in the transparent box; every history walks to the limit
    assert st["n_coll"] == 0 and st["n_stuck"] == len(runs) and st["n_lost"] == 0
    assert np.all(tr["n_seg"] == SEG_LIMIT)
    n, worst = G.compare(runs, o.rays())
    assert n == 919
    assert worst <= TOL, f"largest crossing difference {worst:.3e} cm"
