"""Serving form: continuous batching of requests.

Requests that arrive while others are in flight are admitted as slots free
up and share the particle bank; each request's element tally must be the
same alone and in the mix (1e-12 relative: only the FP64 summation order
of the atomics differs), and equal to mc_run on the same source and seed.
"""
import numpy as np
import pytest

from macaw_gb300 import Tracker, problems
from macaw_gb300._lib import MC_PREC_FP64, MC_PREC_MIXED, MC_SRC_MONO, MC_SRC_POINT
from macaw_gb300.serve import Job, Server, poisson_jobs, run_stream

pytestmark = pytest.mark.gpu


def close(a, b, rtol=1e-12):
    nz = b != 0
    return np.all(a[~nz] == 0) and np.all(np.abs(a[nz] - b[nz]) <= rtol * np.abs(b[nz]))


@pytest.fixture(scope="module")
def probs():
    return [problems.cube_problem(n=8, L=8.0, n_nuc=4, n_pts=2000),
            problems.lattice_problem(nx=3, ny=3, nz=3, height=6.0, n_pts=2000)]


JOBS = [Job(0, 3000, 11, (4.0, 4.0, 4.0), 1.0e6), Job(0, 700, 12, (2.0, 5.0, 3.0), 2.0e5),
        Job(1, 2500, 13, (1.9, 1.9, 3.0), 5.0e5), Job(0, 5000, 14, (6.0, 6.5, 1.5), 3.0e6),
        Job(1, 1200, 15, (1.2, 2.5, 2.0), 1.0e3), Job(0, 1500, 16, (3.3, 3.3, 3.3), 7.0e6)]


def drain(server, keys):
    for _ in range(100000):
        if server.idle():
            break
        server.step()
    assert server.idle()
    return {k: server.result(k) for k in keys}


@pytest.mark.parametrize("precision", [MC_PREC_FP64, MC_PREC_MIXED])
def test_results_are_the_same_alone_and_in_the_mix(probs, precision):
    mix = Server(probs, precision=precision, bank=2048, max_slots=2)  # fewer slots than requests
    keys = [mix.submit(j) for j in JOBS]
    together = drain(mix, keys)
    mix.close()
    for key, job in zip(keys, JOBS):
        alone = Server(probs, precision=precision, bank=2048, max_slots=1)
        k = alone.submit(job)
        ref = drain(alone, [k])[k]
        alone.close()
        assert ref.sum() > 0
        assert close(together[key], ref), f"request {job} differs alone vs in the mix"


def test_fp64_request_equals_mc_run(probs):
    job = JOBS[3]
    srv = Server(probs, precision=MC_PREC_FP64, bank=4096, max_slots=3)
    k = srv.submit(job)
    got = drain(srv, [k])[k]
    srv.close()
    with Tracker(0) as t:
        t.load(probs[0])
        t.set_source(problems.Source(space=MC_SRC_POINT, energy=MC_SRC_MONO, point=job.point, mono_E=job.energy))
        t.run(job.n_histories, seed=job.seed, precision=MC_PREC_FP64)
        assert close(got, t.tally())


def test_poisson_stream_completes(probs):
    srv = Server(probs, precision=MC_PREC_MIXED, bank=8192, max_slots=4)
    jobs = poisson_jobs(probs, rate=200.0, duration=0.2, hist_range=(1e3, 2e4))
    rep = run_stream(srv, jobs)
    srv.close()
    assert rep["requests"] == len(jobs) and rep["p99_ms"] >= rep["p50_ms"] > 0


def test_admitted_requests_overlap_on_the_device(probs):
    """Requests admitted together run together: after one step, several are
    active in one context's bank at once."""
    srv = Server(probs[:1], precision=MC_PREC_FP64, bank=4096, max_slots=3)
    keys = [srv.submit(Job(0, 200_000, 20 + k, (4.0, 4.0, 4.0), 1.0e6)) for k in range(3)]
    srv.step()
    queued, active, free = srv.status(0)
    assert active == 3 and queued == 0 and free == 0
    drain(srv, keys)
    srv.close()


def test_budget_admission_loads_and_evicts(probs):
    """With an HBM budget that holds one problem at a time, requests for the
    other problem wait, the idle problem is evicted and the other loaded;
    every result equals the request run alone."""
    from macaw_gb300.serve import footprint
    budget = max(footprint(p, 2048, 1) for p in probs) + 1024
    srv = Server(probs, precision=MC_PREC_FP64, bank=2048, max_slots=1, hbm_budget=budget, preload=False)
    keys = [srv.submit(j) for j in JOBS]
    together = drain(srv, keys)
    assert srv.loads >= 2 and srv.evictions >= 1
    assert srv.peak_bytes <= budget
    srv.close()
    for key, job in zip(keys, JOBS):
        alone = Server(probs, precision=MC_PREC_FP64, bank=2048, max_slots=1)
        k = alone.submit(job)
        ref = drain(alone, [k])[k]
        alone.close()
        assert close(together[key], ref), f"request {job} differs under eviction"
