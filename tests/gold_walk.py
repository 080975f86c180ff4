"""Straight runs of the reference's gold rays, and their comparison with a walk.

The gold file test/tests/study/gold/openmc_study_rays.e (MaCaw's `study_run`
test on the mesh of test/tests/study/openmc_study.i: 5 x 5 x 1 HEX8 over
[-5, 5]^3, ReflectRayBC on every side) stores every segment of rays 60-89
with its start and end point (fixture openmc_study_rays_points.npz, made by
tests/golden/make_golden.py).  A segment that draws exactly one tracking
number and keeps its energy holds no collision (CollisionKernel.C:150 draws
once per segment; a collision draws more), so between two collisions a ray
is pure geometry: straight chords through the hexes, crossing points on the
hex faces, specular reflections on the box walls.

gold_runs() cuts each ray into maximal runs of such collision-free segments.
A run's first segment starts on a face (the end of the previous segment);
its midpoint and the direction of the run's first straight stretch give a
source site that reproduces the run without the physics.  Every end point of
the run's segments is a hex-face crossing or a wall reflection.

hex_crossings() keeps, of a tet walk's recorded segment end points, those on
a hex face or a box wall (the Kuhn tets also cross the hexes' internal
diagonal faces, which the HEX8 trace does not have).
"""
from __future__ import annotations

import numpy as np

M64 = 2**64
MULT, ADD = 6364136223846793005, 1442695040888963407
HEX_XY = np.array([-5.0, -3.0, -1.0, 1.0, 3.0, 5.0])
HEX_Z = np.array([-5.0, 5.0])
ON_FACE = 1e-9  # a point within this distance of a hex plane lies on it


def step(s: int) -> int:
    return (MULT * s + ADD) % M64


def one_draw(seed_a: float, seed_b: float) -> bool:
    """The tracking state went from seed_a to seed_b by exactly one draw
    (states stored as doubles: the reference resumes from the stored double)."""
    return float(step(int(seed_a))) == seed_b


def gold_runs(g: dict) -> list[dict]:
    rid, inter, E, trk = g["ray_id"], g["intersections"], g["energy"], g["seed_tracking"]
    S, T = g["start"], g["end"]
    runs = []
    for r in np.unique(rid):
        idx = np.where(rid == r)[0]
        idx = idx[np.argsort(inter[idx])]
        clean = [False] + [E[b] == E[a] and one_draw(trk[a], trk[b]) for a, b in zip(idx[:-1], idx[1:])]
        j = 0
        while j < idx.size:
            if not clean[j]:
                j += 1
                continue
            k = j
            while j < idx.size and clean[j]:
                j += 1
            seg = idx[k:j]
            # first straight stretch: up to the first segment ending on a wall
            last = seg[-1]
            for q in seg:
                if np.any(np.isclose(np.abs(T[q]), 5.0, rtol=0.0, atol=ON_FACE)):
                    last = q
                    break
            d = T[last] - S[seg[0]]
            runs.append({"ray": int(r), "segments": seg, "site": 0.5 * (S[seg[0]] + T[seg[0]]),
                         "dir": d / np.linalg.norm(d), "points": T[seg]})
    return runs


def on_hex_face(p: np.ndarray) -> bool:
    return bool(np.min(np.abs(p[0] - HEX_XY)) <= ON_FACE or np.min(np.abs(p[1] - HEX_XY)) <= ON_FACE
                or np.min(np.abs(p[2] - HEX_Z)) <= ON_FACE)


def hex_crossings(ends: np.ndarray) -> np.ndarray:
    """End points on a hex face or box wall, in walk order; a point that
    repeats the previous one (a crossing through a hex edge, where the tet
    walk ends two segments at the same place) is kept once."""
    out = []
    for p in ends:
        if on_hex_face(p) and not (out and np.max(np.abs(p - out[-1])) <= ON_FACE):
            out.append(p)
    return np.array(out).reshape(-1, 3)


def compare(runs: list[dict], rays: np.ndarray) -> tuple[int, float]:
    """Matches each run against the recorded ray of the history started at
    its site (history i = run i); returns (points compared, max abs error).
    Raises AssertionError on a missing or extra crossing."""
    n_pts, worst = 0, 0.0
    for i, run in enumerate(runs):
        seg = rays[rays["id"] == i + 1]
        seg = seg[np.argsort(seg["segment"])]
        got = hex_crossings(seg["end"])
        want = run["points"]
        assert got.shape[0] >= want.shape[0], \
            f"run {i} (ray {run['ray']}): {got.shape[0]} crossings recorded, gold has {want.shape[0]}"
        err = np.max(np.abs(got[:want.shape[0]] - want))
        assert err < 1e-6, f"run {i} (ray {run['ray']}): crossing off by {err}"
        n_pts += want.shape[0]
        worst = max(worst, float(err))
    return n_pts, worst


def sites(runs: list[dict], E: float = 1.0e6) -> np.ndarray:
    out = np.zeros((len(runs), 8))
    for i, r in enumerate(runs):
        out[i, :3] = r["site"]
        out[i, 3:6] = r["dir"]
        out[i, 6] = E
        out[i, 7] = 1.0
    return out
