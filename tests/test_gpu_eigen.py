"""k-eigenvalue generations on the GPU against the oracle.

FP64 form, event and history execution: every generation's keff
estimators, running keff and its deviation, site count, segment and
collision counts equal the oracle's bit for bit; so do the last
generation's sorted fission bank and the resampled source of the next one
(OpenMCStudy.C:297-607 restated: bank sort, synchronize_bank).  The bank
resampling is exercised longer and shorter than n_particles.  Mixed form:
keff within the statistics of the FP64 run.  Active-generation tallies
match the oracle's within atomic summation order.
"""
import numpy as np
import pytest

from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import MC_MODE_EVENT, MC_MODE_HISTORY, MC_PREC_FP64, MC_PREC_MIXED, MC_TALLY_SUM, MCError

from oracle import oracle as O

pytestmark = pytest.mark.gpu

N = 5000
FIELDS = ("k_generation", "k_collision", "k_absorption", "keff", "keff_std", "leakage", "n_sites", "n_seg",
          "n_coll")


@pytest.fixture(scope="module")
def small():
    return problems.eigen_lattice_problem(nx=5, ny=5, nz=6, height=15.0, n_pts=3000)


@pytest.fixture(scope="module")
def ref(small):
    return O.Oracle(small).eigen(N, 4, 2, seed=3, threads=16, tally=True)


def _src_rows(sites):
    return np.stack([sites[f] for f in ("x", "y", "z", "u", "v", "w", "E", "wgt")], axis=1)


def _same_bank(a, b):
    for f in ("x", "y", "z", "u", "v", "w", "E", "wgt", "parent", "progeny"):
        assert np.array_equal(a[f], b[f]), f


@pytest.mark.parametrize("mode", [MC_MODE_EVENT, MC_MODE_HISTORY])
def test_fp64_generations_match_the_oracle(small, ref, mode):
    g_ref, src_ref, bank_ref, tally_ref, _ = ref
    with Tracker(0) as t:
        t.load(small)
        g = t.eigen(N, 4, 2, seed=3, mode=mode, precision=MC_PREC_FP64, bank_size=2048, max_seg=32)
        bank = t.fission_bank()
        src = t.eigen_source(N)
        tally = t.tally(MC_TALLY_SUM)
        assert t.batches_done() == 2
    for f in FIELDS:
        assert np.array_equal(g[f], g_ref[f]), (f, g[f], g_ref[f])
    _same_bank(bank, bank_ref)
    assert np.array_equal(_src_rows(src), src_ref)
    nz = tally_ref != 0
    assert np.all(tally[~nz] == 0)
    assert np.allclose(tally[nz], tally_ref[nz], rtol=1e-12, atol=0)


@pytest.mark.parametrize("keff0", [0.4, 3.0])
def test_resampling_longer_and_shorter_banks(small, keff0):
    n = 3000
    g_ref, src_ref, bank_ref, _, _ = O.Oracle(small).eigen(n, 1, 0, seed=11, keff0=keff0, threads=16)
    with Tracker(0) as t:
        t.load(small)
        g = t.eigen(n, 1, 0, seed=11, keff0=keff0, bank_size=1024, max_seg=16, sort_queue=3)
        bank = t.fission_bank()
        src = t.eigen_source(n)
    assert (bank.size > n) if keff0 < 1 else (bank.size < n)
    for f in FIELDS:
        assert np.array_equal(g[f], g_ref[f]), f
    _same_bank(bank, bank_ref)
    assert np.array_equal(_src_rows(src), src_ref)


def test_initial_source_from_the_host(small):
    n = 2000
    with Tracker(0) as t:
        t.load(small)
        sites = t.sample_sites(n, seed=21)
        sites["E"] = 1.0e6
        g = t.eigen(n, 2, 1, seed=4, initial_source=sites)
    ref = O.Oracle(small).eigen(n, 2, 1, seed=4, threads=16, initial_source=_src_rows(sites))[0]
    for f in FIELDS:
        assert np.array_equal(g[f], ref[f]), f


def test_mixed_keff_agrees_with_fp64(small):
    n = 20000
    with Tracker(0) as t:
        t.load(small)
        gd = t.eigen(n, 8, 3, seed=5, precision=MC_PREC_FP64, max_seg=32)
        gm = t.eigen(n, 8, 3, seed=5, precision=MC_PREC_MIXED, max_seg=64)
    kd, km = gd["keff"][-1], gm["keff"][-1]
    sd = max(gd["keff_std"][-1], gm["keff_std"][-1])
    assert abs(km - kd) < 4 * sd + 0.01, (kd, km, sd)
    assert np.all(gm["n_sites"] > 0)


def test_fixed_source_with_fission_data_matches_the_oracle(small):
    """Fission sites are drawn and dropped in fixed-source runs: the FP64
    histories stay bit-identical to the oracle's."""
    n = 4000
    _, tr_ref, _, _ = O.Oracle(small).run(n, seed=2, threads=16)
    for mode in (MC_MODE_EVENT, MC_MODE_HISTORY):
        with Tracker(0) as t:
            t.load(small)
            t.run(n, seed=2, mode=mode, precision=MC_PREC_FP64, traces=True, bank_size=1024, max_seg=32)
            tr = t.traces(n)
        for f in ("hash", "status", "n_seg", "n_coll", "elem", "E", "x", "y", "z"):
            assert np.array_equal(tr[f], tr_ref[f]), (mode, f)


def test_eigen_errors(small):
    with Tracker(0) as t:
        t.load(small)
        with pytest.raises(MCError):
            t.eigen(1000, 2, 0, capacity=10)  # fission bank full
        with pytest.raises(MCError):
            t.eigen(1000, 2, 2)  # inactive must be below batches
    plain = problems.lattice_problem(nx=3, ny=3, nz=2, height=5.0, n_pts=500)
    with Tracker(0) as t:
        t.load(plain)
        with pytest.raises(MCError):
            t.eigen(100, 1, 0)  # nothing fissionable


def test_eigen_with_a_collision_tally_and_energy_bins(small):
    """Active generations score an OpenMCTally definition (collision
    estimator, four scores, energy filter) as fixed-source runs do."""
    from macaw_gb300._lib import (MC_EST_COLLISION, MC_SCORE_ABSORPTION, MC_SCORE_FLUX, MC_SCORE_SCATTER,
                                  MC_SCORE_TOTAL)
    d = problems.TallyDef(MC_EST_COLLISION, (MC_SCORE_FLUX, MC_SCORE_TOTAL, MC_SCORE_SCATTER, MC_SCORE_ABSORPTION),
                          np.array([1.0e-5, 1.0, 1.0e3, 1.0e6, 2.0e7]))
    small.tally = d
    try:
        g_ref, _, _, t_ref, _ = O.Oracle(small).eigen(3000, 3, 1, seed=6, threads=16, tally=True)
        with Tracker(0) as t:
            t.load(small)
            g = t.eigen(3000, 3, 1, seed=6, bank_size=1024, max_seg=16)
            tally = t.tally(MC_TALLY_SUM)
    finally:
        small.tally = None
    for f in FIELDS:
        assert np.array_equal(g[f], g_ref[f]), f
    assert tally.size == t_ref.size == small.n_tet * 4 * 4
    nz = t_ref != 0
    assert np.all(tally[~nz] == 0) and np.allclose(tally[nz], t_ref[nz], rtol=1e-12, atol=0)


def test_eigen_in_two_d_mode():
    """2-D eigenvalue generations (CollisionKernel z_coord): sites stay in the
    plane and the generations equal the oracle's."""
    p = problems.lattice_2d_problem(nx=5, ny=5, n_pts=3000)
    for k in p.materials[0].nuclides:
        problems.add_fission(p.nuclides[int(k)], 2.43, 0.6)
    for n_ in p.nuclides:
        n_.sig_s = n_.sig_s + 2.0
        n_.sig_t = n_.sig_t + 2.5
        if n_.nu_sig_f is not None:
            n_.nu_sig_f = (2.43 * 0.6) * (n_.sig_t - n_.sig_s)
    for b in (1, 2, 3, 4):
        p.bcs[b] = 1
    g_ref, src_ref, bank_ref, _, _ = O.Oracle(p).eigen(2000, 3, 1, seed=2, threads=16)
    with Tracker(0) as t:
        t.load(p)
        g = t.eigen(2000, 3, 1, seed=2, bank_size=1024)
        bank = t.fission_bank()
        src = t.eigen_source(2000)
    for f in FIELDS:
        assert np.array_equal(g[f], g_ref[f]), f
    _same_bank(bank, bank_ref)
    assert np.all(bank["z"] == p.z_2d)
    assert np.array_equal(_src_rows(src), src_ref)
