"""The oracle's random-number scheme against the reference's golden file.

MaCaw's only gold file (test/tests/study/gold/openmc_study_rays.e, the
`study_run` Exodiff test) stores, per traced segment of rays 60..89 (batch 3
of 30 particles), the OpenMC seeds as doubles in the ray aux data.  The
fixture tests/golden/openmc_study_rays_seeds.npz holds those columns
(made by tests/golden/make_golden.py).  What they pin:

* the LCG state step: between two segments without a collision exactly one
  random number is drawn (CollisionKernel.C:150), and the reference stores
  the state as a double in between (CollisionKernel.C:132-134,157-159), so
  seed_{k+1} == double(step(uint64(seed_k)));
* the per-history seeds: stream s of particle id starts at
  future_seed(id * 152917, master + s) with master seed 1 (ids 61..90 for
  batch 3: OpenMC ids are global across batches);
* the first segment draws one number from the stream-0 seed.
"""
import numpy as np
import pytest

from oracle import oracle as O

M64 = 2**64
MULT, ADD = 6364136223846793005, 1442695040888963407


def step(s: int) -> int:
    return (MULT * s + ADD) % M64


@pytest.fixture(scope="module")
def gold(golden_dir):
    return dict(np.load(golden_dir / "openmc_study_rays_seeds.npz"))


def test_oracle_step_matches_python_step():
    s = 12345
    for _ in range(100):
        _, s2 = O.prn(s)
        assert s2 == step(s)
        s = s2


def test_skip_ahead_equals_repeated_steps():
    for n in (0, 1, 2, 3, 17, 152917, 1000003):
        s = 987654321
        for _ in range(min(n, 2000)):
            s = step(s)
        if n <= 2000:
            assert O.future_seed(n, 987654321) == s
    # composition: future(a+b) == future(a) then future(b)
    a, b, s0 = 123456789, 987654, 42
    assert O.future_seed(a + b, s0) == O.future_seed(b, O.future_seed(a, s0))


def _steps(a: float, b: float, limit: int = 64) -> int:
    """Draws that take the state stored as double a to the one stored as b
    (0 when b is not reached within limit draws)."""
    s = int(a)
    for k in range(1, limit + 1):
        s = step(s)
        if float(s) == b:
            return k
    return 0


def test_gold_segment_to_segment_steps(gold):
    rid, inter, E, trk = gold["ray_id"], gold["intersections"], gold["energy"], gold["seed_tracking"]
    one = same_E = 0
    for r in np.unique(rid):
        idx = np.where(rid == r)[0]
        idx = idx[np.argsort(inter[idx])]
        for a, b in zip(idx[:-1], idx[1:]):
            assert inter[b] == inter[a] + 1
            if E[a] != E[b]:
                continue  # a scatter: its draws depend on the physics
            same_E += 1
            k = _steps(trk[a], trk[b])
            assert k > 0, f"ray {r}: next seed not reachable from the previous one"
            if k == 1:
                one += 1
            else:
                # more than the one distance draw without an energy change:
                # only an absorption, which ends the ray, does that
                assert b == idx[-1], f"ray {r}, segment {inter[b]}: {k} draws but the ray goes on"
    assert same_E == 939
    assert one == 919  # the collision-free segments (tests/test_gold_walk.py walks them)


# Rays whose first segment draws more than the one distance number: ray 64
# is absorbed in its first (and only) segment after 4 draws; rays 60, 61, 75
# and 76 collide in their first segment and sample fission there (their
# tracking state is not reachable by single-stream steps, and 60 and 76 also
# moved their URR stream by 9 draws).
FIRST_SEGMENT_COLLIDES = {60, 61, 64, 75, 76}


def test_gold_initial_seeds(gold):
    rid, src, urr, trk = gold["ray_id"], gold["seed_source"], gold["seed_urr"], gold["seed_tracking"]
    rays = np.unique(rid)
    assert rays.size == 30
    collided = set()
    for r in rays:
        idx = np.where(rid == r)[0]
        pid = int(r) + 1  # batch 3 of 30 particles: ids 61..90
        # stream 1 is never advanced on this path: every segment carries the initial seed
        assert np.all(src[idx] == float(O.init_seed(pid, 1, 1)))
        k = _steps(float(O.init_seed(pid, 1, 0)), trk[idx[0]])
        if k == 1:
            # one draw in the first segment: no collision, so the URR stream
            # is still at its initial seed
            assert urr[idx[0]] == float(O.init_seed(pid, 1, 2)), f"ray {r}"
        else:
            collided.add(int(r))
    assert collided == FIRST_SEGMENT_COLLIDES
    r64 = np.where(rid == 64)[0]
    assert r64.size == 1 and _steps(float(O.init_seed(65, 1, 0)), trk[r64[0]]) == 4
    for r in (60, 76):
        i0 = np.where(rid == r)[0][0]
        assert _steps(float(O.init_seed(r + 1, 1, 2)), urr[i0]) == 9
