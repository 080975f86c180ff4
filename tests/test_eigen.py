"""k-eigenvalue mode on the oracle: estimators, bank order, resampling.

OpenMC's eigenvalue mode as OpenMCStudy runs it (one generation per batch;
src/userobjects/OpenMCStudy.C:297-607): fission sites banked at collisions,
the bank sorted by (parent id, progeny index), resampled to exactly
n_particles sites (synchronizeBanks / synchronize_bank), keff from the
track-length estimator (CollisionKernel.C:153-154).  These checks hold
exactly or statistically:
  - the three keff estimators (track length, collision, absorption) agree;
  - the bank is in (parent, progeny) order with progeny 0..k-1 per parent;
  - the next source equals an independent restatement of synchronize_bank
    (below, in Python, from the sorted bank and the generation's stream),
    for banks longer and shorter than n_particles;
  - keff follows OpenMC's calculate_average_keff over the generations;
  - generations do not depend on the number of threads;
  - a fissionable nuclide changes fixed-source histories only through the
    draws of the sites it samples and drops.
"""
import numpy as np
import pytest

from macaw_gb300 import problems

from oracle import oracle as O


@pytest.fixture(scope="module")
def small():
    return problems.eigen_lattice_problem(nx=5, ny=5, nz=6, height=15.0, n_pts=3000)


def _sync_restated(bank, n, seed, gen):
    """OpenMC synchronize_bank on one rank: per sorted site, n // m copies
    when fewer than n sites were banked, plus one when the next draw of the
    generation's tracking stream (id = generation number, 1-based) is below
    p = needed / m; cut at n, or completed from the end of the bank."""
    m = bank.size
    needed = n % m if m < n else n
    p = needed / m
    s = O.init_seed(gen + 1, seed, 0)
    out = []
    for i in range(m):
        if m < n:
            out += [i] * (n // m)
        xi, s = O.prn(s)
        if xi < p:
            out.append(i)
    out = out[:n]
    need = n - len(out)
    out += [max(0, m - need + j) for j in range(need)]
    b = bank[np.array(out, np.int64)]
    return np.stack([b[f] for f in ("x", "y", "z", "u", "v", "w", "E", "wgt")], axis=1)


def test_estimators_agree_and_bank_is_sorted(small):
    o = O.Oracle(small)
    g, src, bank, _, _ = o.eigen(6000, 4, 1, seed=3, threads=8)
    for r in g[1:]:
        assert abs(r["k_collision"] / r["k_generation"] - 1) < 0.05
        assert abs(r["k_absorption"] / r["k_generation"] - 1) < 0.08
    assert 0.8 < g["k_generation"][-1] < 1.6
    assert bank.size == g["n_sites"][-1]
    # (parent, progeny) order; progeny numbers each parent's sites 0..k-1
    assert np.all(np.diff(bank["parent"]) >= 0)
    first = np.r_[True, bank["parent"][1:] != bank["parent"][:-1]]
    starts = np.flatnonzero(first)
    cnt = np.diff(np.r_[starts, bank.size])
    expect = np.concatenate([np.arange(c) for c in cnt])
    assert np.array_equal(bank["progeny"], expect)
    # last generation's parents are its histories
    assert bank["parent"].min() >= 3 * 6000 + 1 and bank["parent"].max() <= 4 * 6000
    assert np.all(bank["wgt"] == 1.0)
    assert np.allclose(bank["u"] ** 2 + bank["v"] ** 2 + bank["w"] ** 2, 1.0, atol=1e-12)
    assert src.shape == (6000, 8)


@pytest.mark.parametrize("keff0", [0.4, 1.0, 3.0])
def test_resampling_matches_synchronize_bank(small, keff0):
    """keff0 far from k makes the first bank about n*k/keff0 sites: longer
    than n (keff0 0.4), near n, or shorter (keff0 3.0: copies + draws)."""
    n, seed = 3000, 11
    o = O.Oracle(small)
    g, src, bank, _, _ = o.eigen(n, 1, 0, seed=seed, keff0=keff0, threads=8)
    assert bank.size == g["n_sites"][0]
    if keff0 == 0.4:
        assert bank.size > n
    if keff0 == 3.0:
        assert bank.size < n
    assert np.array_equal(src, _sync_restated(bank, n, seed, 0))


def test_keff_follows_calculate_average_keff(small):
    o = O.Oracle(small)
    g, _, _, _, _ = o.eigen(2000, 6, 2, seed=5, threads=8)
    kg = g["k_generation"]
    assert np.array_equal(g["keff"][:2], kg[:2])  # inactive: the generation's own estimate
    for i in range(2, 6):
        a = kg[2:i + 1]
        n = a.size
        s0 = 0.0
        s1 = 0.0
        for v in a:
            s0 += v
            s1 += v * v
        mean = s0 / n
        assert g["keff"][i] == mean
        if n > 1:
            assert g["keff_std"][i] == np.sqrt((s1 / n - mean * mean) / (n - 1))


def test_generations_do_not_depend_on_threads(small):
    """Per-history estimator sums, the fixed-order reduction and the
    ordered bank make every generation independent of the thread count."""
    o = O.Oracle(small)
    a = o.eigen(2000, 3, 1, seed=9, threads=8)
    b = o.eigen(2000, 3, 1, seed=9, threads=3)
    assert np.array_equal(a[0], b[0])
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[2], b[2])


def test_fixed_source_fission_sites_are_drawn_and_dropped(small):
    """With fission data a fixed-source history draws its sites' numbers at
    collisions with fissionable nuclides; without it, not.  Histories that
    never collide with a fuel nuclide are unchanged."""
    p = problems.eigen_lattice_problem(nx=5, ny=5, nz=6, height=15.0, n_pts=3000)
    _, tr_f, st_f, _ = O.Oracle(p).run(3000, seed=2, threads=8)
    for n in p.nuclides:
        n.nu_sig_f = None
    _, tr_n, st_n, _ = O.Oracle(p).run(3000, seed=2, threads=8)
    same = tr_f["hash"] == tr_n["hash"]
    assert 0 < same.sum() < same.size
    assert np.all(tr_f["n_coll"][~same] > 0)
    assert np.all(tr_f["n_coll"][(tr_f["n_coll"] == 0)] == tr_n["n_coll"][(tr_f["n_coll"] == 0)])
