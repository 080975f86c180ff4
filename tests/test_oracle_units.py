"""Unit and statistical checks of the CPU oracle (no GPU)."""
import numpy as np
import pytest

from macaw_gb300 import problems
from macaw_gb300._lib import MC_BC_REFLECT, MC_SRC_BOX, MC_SRC_MONO
from oracle import oracle as O


def ulp_err(a: float, b: float) -> float:
    return abs(a - b) / np.spacing(abs(b)) if b != 0 else abs(a)


def test_log_accuracy_and_specials():
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.random(20000), np.exp(rng.uniform(-700, 700, 20000)),
                         1.0 + rng.uniform(-1e-6, 1e-6, 2000), [1.0, 2.0, 0.5, 1e-300, 5e-324, 1.7e308]])
    worst = max(ulp_err(O.log(float(x)), float(np.log(x))) for x in xs if x > 0)
    assert worst <= 2.0, worst
    assert O.log(1.0) == 0.0
    assert O.log(0.0) == -np.inf
    assert np.isnan(O.log(-1.0))
    assert O.log(np.inf) == np.inf


def test_quotient_within_an_ulp_of_the_ieee_division():
    """The walks' num / den (float reciprocal, one Newton step, residual
    correction) stays within an ulp of the correctly rounded quotient, and
    a denominator outside the float range [2^-100, 2^100] takes the IEEE
    division itself."""
    rng = np.random.default_rng(7)
    num = rng.uniform(-1.0, 1.0, 40000) * np.exp(rng.uniform(-40, 40, 40000))
    den = rng.uniform(0.0, 1.0, 40000) * np.exp(rng.uniform(-60, 60, 40000)) + 1e-300
    worst, exact = 0.0, 0
    for a, b in zip(num, den):
        q, ref = O.quotient(float(a), float(b)), float(a) / float(b)
        worst = max(worst, ulp_err(q, ref))
        exact += q == ref
    assert worst <= 1.0, worst
    assert exact / num.size > 0.99  # correctly rounded but in rare near-midpoint cases
    for b in (2.0 ** -110, 2.0 ** 120, 3e-320):
        assert O.quotient(1.234, b) == 1.234 / b
    assert O.quotient(0.0, 3.0) == 0.0


def test_prn_range_and_uniformity():
    s = O.init_seed(1, 1, 0)
    v = []
    for _ in range(20000):
        x, s = O.prn(s)
        v.append(x)
    v = np.array(v)
    assert v.min() >= 0.0 and v.max() < 1.0
    assert abs(v.mean() - 0.5) < 0.01
    assert abs(v.var() - 1 / 12) < 0.005


@pytest.fixture(scope="module")
def small_cube():
    return problems.cube_problem(n=6, n_nuc=3, n_pts=3000)


def test_xs_index_matches_searchsorted_on_grid_points(small_cube):
    o = O.Oracle(small_cube)
    E = small_cube.nuclides[1].E
    n = E.size
    probes = np.concatenate([E[1:-1], np.nextafter(E[1:-1], 0), np.nextafter(E[1:-1], np.inf),
                             np.exp(np.random.default_rng(2).uniform(np.log(E[0]), np.log(E[-1]), 3000))])
    for e in probes:
        i, f = o.xs_index(1, float(e))
        j = min(max(int(np.searchsorted(E, e, side="right")) - 1, 0), n - 2)
        assert i == j
        assert 0.0 <= f <= 1.0


def test_macro_xs_matches_numpy_interpolation(small_cube):
    o = O.Oracle(small_cube)
    m = small_cube.materials[0]
    for e in (1e-4, 0.3, 7.0, 2.5e3, 1.1e6, 1.9e7):
        ref = sum(d * np.interp(e, small_cube.nuclides[k].E, small_cube.nuclides[k].sig_t)
                  for k, d in zip(m.nuclides, m.densities))
        assert o.macro_xs(0, e) == pytest.approx(ref, rel=1e-12)


def test_locate_at_shared_vertex_picks_entered_tet():
    p = problems.cube_problem(n=4, L=4.0, n_nuc=1, n_pts=100)
    o = O.Oracle(p)
    nbr, planes = o.mesh_tables()
    x = np.array([2.0, 2.0, 2.0])
    rng = np.random.default_rng(3)
    for _ in range(200):
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        t = o.locate(x, u)
        assert t >= 0
        # a small step along u stays inside the chosen tet
        y = x + 1e-6 * u
        s = planes[t, :, :3] @ y - planes[t, :, 3]
        assert np.all(s <= 1e-12)


def test_adjacency_is_symmetric_and_planes_negated():
    p = problems.lattice_problem(nx=2, ny=2, nz=2, n_pts=100)
    o = O.Oracle(p)
    nbr, planes = o.mesh_tables()
    for t in range(0, p.n_tet, 7):
        for f in range(4):
            nb = nbr[t, f]
            if nb < 0:
                continue
            g = int(np.where(nbr[nb] == t)[0][0])
            assert np.array_equal(planes[nb, g], -planes[t, f])


def _flat_problem(L=10.0, n=5, sig_t=0.5, c=0.5, awr=20.0, reflect=True):
    p = problems.cube_problem(n=n, L=L, n_nuc=1, n_pts=50)
    E = np.geomspace(1e-5, 2e7, 50)
    p.nuclides = [problems.Nuclide(E, np.full(50, sig_t), np.full(50, c * sig_t), awr)]
    p.materials = [problems.Material(1, np.array([0], np.int32), np.array([1.0]))]
    if reflect:
        p.bcs = {b: MC_BC_REFLECT for b in range(6)}
    p.source = problems.Source(space=MC_SRC_BOX, energy=MC_SRC_MONO, box_lo=(0, 0, 0), box_hi=(L, L, L),
                               mono_E=1.0e6)
    return p


def test_infinite_medium_track_length_and_collisions():
    """All-reflective box, constant Sigma_t and scatter ratio c: the mean
    track length per history is 1/Sigma_a and the mean number of
    collisions is 1/(1-c)."""
    sig_t, c = 0.5, 0.5
    o = O.Oracle(_flat_problem(sig_t=sig_t, c=c))
    n = 20000
    tally, tr, st, _ = o.run(n, threads=4)
    assert st["n_leak"] == 0 and st["n_stuck"] == 0 and st["n_lost"] == 0
    assert st["n_absorb"] + st["n_cutoff"] == n
    mean_track = tally.sum() / n
    sig_a = sig_t * (1 - c)
    # track length is exponential-sum distributed with mean 1/sig_a, sd ~ 1/sig_a
    assert abs(mean_track - 1 / sig_a) < 5 * (1 / sig_a) / np.sqrt(n)
    mean_coll = st["n_coll"] / n
    assert abs(mean_coll - 1 / (1 - c)) < 5 * np.sqrt(c) / (1 - c) / np.sqrt(n)


def test_pure_absorber_escape_probability():
    """Point source at the centre of a vacuum cube of pure absorber: the
    escape probability is E[exp(-Sigma R(omega))] over isotropic omega."""
    L, sig = 10.0, 0.2
    p = _flat_problem(L=L, sig_t=sig, c=0.0, reflect=False)
    p.source = problems.Source(energy=MC_SRC_MONO, point=(L / 2, L / 2, L / 2), mono_E=1.0e6)
    o = O.Oracle(p)
    n = 40000
    _, tr, st, _ = o.run(n, threads=4)
    rng = np.random.default_rng(5)
    u = rng.normal(size=(400000, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    R = (L / 2) / np.abs(u).max(axis=1)
    expect = np.exp(-sig * R).mean()
    got = st["n_leak"] / n
    assert abs(got - expect) < 5 * np.sqrt(expect * (1 - expect) / n) + 1e-3


def test_history_accounting_and_determinism(small_cube):
    o = O.Oracle(small_cube)
    t1, tr1, st1, _ = o.run(3000, seed=7, threads=1)
    t2, tr2, st2, _ = o.run(3000, seed=7, threads=4)
    assert np.array_equal(tr1, tr2)
    assert np.allclose(t1, t2, rtol=1e-13, atol=0)
    assert st1 == st2
    total = sum(st1[k] for k in ("n_leak", "n_absorb", "n_cutoff", "n_stuck", "n_lost", "n_badxs"))
    assert total == 3000
    assert st1["n_stuck"] == 0 and st1["n_lost"] == 0
    # a history range is the same whether run alone or inside a larger batch
    _, tr3, _, _ = o.run(1000, first=1000, seed=7)
    assert np.array_equal(tr3, tr1[1000:2000])
