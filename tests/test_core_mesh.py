"""Cylindrical core generator (the batched large-mesh workload's geometry).

The full core (193 assemblies of 17x17 pin cells, radius 180 cm, 400 cm,
about 41M tets) is generated on the GPU tests' host; here a small core of
2x2-pin assemblies checks the construction: conforming adjacency, volume,
block ids, sidesets, pin centres, material draws, and that the oracle
tracks histories through it without losing any.
"""
import numpy as np
import pytest

from macaw_gb300 import problems

from oracle import oracle as O

PITCH, H, R = 1.26, 6.0, 22.0
PINS, NZ, NSEC = 2, 2, 8


@pytest.fixture(scope="module")
def mesh():
    return problems.core_mesh(pins=PINS, nz=NZ, n_sec=NSEC, n_fuel_rings=1, pitch=PITCH, height=H, radius=R)


def _vol(xyz, tv):
    a, b, c, d = (xyz[tv[:, k]] for k in range(4))
    return np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a) / 6.0


def test_pins_blocks_and_volume(mesh):
    xyz, tv, blk, bid, pins = mesh
    assert pins.shape == (193 * PINS * PINS, 2)
    assert set(np.unique(blk)) == set(range(1, 201))
    v = np.abs(_vol(xyz, tv))
    assert v.min() > 0
    # every pin cell is a full square of pitch^2; fuel is an n_sec-gon
    pin_cell = v[(blk >= 1) & (blk <= 195)].sum()
    assert pin_cell == pytest.approx(193 * PINS * PINS * PITCH**2 * H, rel=1e-12)
    gon = NSEC / 2 * 0.41**2 * np.sin(2 * np.pi / NSEC)
    for b in (1, 97, 193):
        assert v[blk == b].sum() == pytest.approx(PINS * PINS * gon * H, rel=1e-12)
    # the reflector is made of whole cells inside the radius
    refl = v[blk >= 196].sum() / (PITCH**2 * H)
    assert abs(refl - round(refl)) < 1e-9 and refl > 0
    r = np.hypot(xyz[:, 0], xyz[:, 1])
    assert r.max() <= R
    assert np.all((xyz[:, 2] >= 0) & (xyz[:, 2] <= H))


def test_adjacency_conforms_and_sidesets(mesh):
    xyz, tv, blk, bid, pins = mesh
    p = problems.Problem("core-small", xyz, tv, blk, bid, [problems.make_nuclide(1, 0, 100)],
                         [problems.Material(1, np.array([0], np.int32), np.array([0.01]))],
                         np.arange(1, 201, dtype=np.int32), np.ones(200, np.int32),
                         problems.Source(point=(0.0, 0.0, H / 2)), {b: 0 for b in range(7)})
    o = O.Oracle(p)
    nbr, planes = o.mesh_tables()
    inner = nbr >= 0
    t, f = np.nonzero(inner)
    back = nbr[t, f]
    # the neighbour across each interior face points back
    assert np.all((nbr[back] == t[:, None]).any(axis=1))
    # boundary faces: z = 0 (sideset 0), z = H (sideset 5), radial staircase (6)
    tb, fb = np.nonzero(~inner)
    ids = bid[tb, fb]
    assert set(np.unique(ids)) == {0, 5, 6}
    fv = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])
    z = xyz[tv[tb[:, None], fv[fb]], 2]
    assert np.all(z[ids == 0] == 0.0) and np.all(z[ids == 5] == H)
    rad = ids == 6
    assert np.all(z[rad].min(axis=1) < z[rad].max(axis=1))  # radial faces are vertical
    # a closed surface: the outward area vectors of the boundary sum to zero
    vtx = xyz[tv[tb[:, None], fv[fb]]]
    opp = xyz[tv[tb, fb]]  # the vertex opposite face f is vertex f
    an = 0.5 * np.cross(vtx[:, 1] - vtx[:, 0], vtx[:, 2] - vtx[:, 0])
    an *= -np.sign(np.einsum("ij,ij->i", an, opp - vtx[:, 0]))[:, None]
    area = np.linalg.norm(an, axis=1).sum()
    assert np.abs(an.sum(axis=0)).max() < 1e-9 * area


def test_material_draws_are_deterministic():
    lo, hi = 5, 40
    cnt = [lo + problems._splitmix(20240611 * 1000003 + b) % (hi - lo + 1) for b in range(1, 201)]
    assert min(cnt) >= lo and max(cnt) <= hi and len(set(cnt)) > 20
    assert problems._splitmix(0) == 0xE220A8397B1DCDAF


def test_oracle_tracks_through_the_small_core():
    p = problems.core_problem(pins=PINS, nz=NZ, height=H, radius=R, n_pool=48, n_pts=500, max_peaks=6)
    assert len(p.materials) == 200
    assert all(5 <= m.nuclides.size <= 40 and np.unique(m.nuclides).size == m.nuclides.size for m in p.materials)
    o = O.Oracle(p)
    tally, tr, st, _ = o.run(2000, seed=3, threads=4)
    assert st["n_stuck"] == 0 and st["n_lost"] == 0 and st["n_badxs"] == 0
    assert sum(st[k] for k in ("n_leak", "n_absorb", "n_cutoff")) == 2000
    assert tally.sum() > 0
