"""Serving form: a request loop over preloaded fixed-source problems.

Each preloaded problem (mesh + cross sections) lives resident in its own
context with its own CUDA stream.  Requests (problem, source point,
energy, history count, seed) are queued as they arrive; the C ABI's
serving calls (mc_serve_*) admit them into tally slots of their problem's
context and run them through that context's continuous event pipeline, so
requests on one problem share a particle bank and requests on different
problems overlap on separate streams.  The number of slots each problem
gets is set by an HBM budget: the resident footprint of every problem plus
one n_tet tally per slot must fit.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from ._lib import MC_PREC_FP64, MC_PREC_MIXED, MC_SRC_MONO, MC_SRC_POINT, MCError, Request, SourceDesc, lib
from .problems import Problem, Source
from .tracker import Tracker


@dataclass
class Job:
    problem: int
    n_histories: int
    seed: int
    point: tuple
    energy: float
    arrival: float = 0.0


def footprint(p: Problem, bank: int) -> int:
    """Resident bytes of a problem: mesh tables, cross sections, bank."""
    return p.footprint_bytes() + bank * 250


class Server:
    def __init__(self, problems: list[Problem], device: int = 0, precision: int = MC_PREC_MIXED,
                 hbm_budget: int = 64 << 30, bank: int = 262144, max_seg: int = 64, max_slots: int = 8,
                 iterations: int = 4):
        self.iterations = iterations
        self.trackers: list[Tracker] = []
        self.slots: list[int] = []
        resident = sum(footprint(p, bank) for p in problems)
        if resident > hbm_budget:
            raise MCError(1, f"problems need {resident} bytes, over the HBM budget of {hbm_budget}")
        spare = hbm_budget - resident
        for p in problems:
            t = Tracker(device)
            t.load(p)
            per_slot = t.tally_size() * 8
            n_slots = int(max(1, min(max_slots, spare // (len(problems) * per_slot))))
            t._ck(lib.mc_serve_open(t._h, n_slots, bank, precision, max_seg), "mc_serve_open")
            self.trackers.append(t)
            self.slots.append(n_slots)
        self.pending: dict[tuple, float] = {}  # (problem, ticket) -> submit time
        self.done: dict[tuple, float] = {}     # (problem, ticket) -> completion time

    def submit(self, job: Job) -> tuple:
        t = self.trackers[job.problem]
        r = Request()
        r.n_histories = job.n_histories
        r.seed = job.seed
        r.source.space = MC_SRC_POINT
        r.source.energy = MC_SRC_MONO
        r.source.point[:] = job.point
        r.source.mono_E = job.energy
        tk = C.c_int64()
        t._ck(lib.mc_serve_submit(t._h, C.byref(r), C.byref(tk)), "mc_serve_submit")
        key = (job.problem, tk.value)
        self.pending[key] = time.perf_counter()
        return key

    def step(self) -> list[tuple]:
        """Admit and launch on every problem, then collect finished requests."""
        busy = []
        for i, t in enumerate(self.trackers):
            q, a = C.c_int32(), C.c_int32()
            t._ck(lib.mc_serve_status(t._h, C.byref(q), C.byref(a), None), "mc_serve_status")
            if q.value or a.value:
                t._ck(lib.mc_serve_step(t._h, self.iterations), "mc_serve_step")
                busy.append(i)
        finished = []
        buf = (C.c_int64 * 256)()
        for i in busy:
            t = self.trackers[i]
            n = C.c_int32()
            t._ck(lib.mc_serve_poll(t._h, buf, 256, C.byref(n)), "mc_serve_poll")
            now = time.perf_counter()
            for k in range(n.value):
                key = (i, buf[k])
                self.done[key] = now
                self.pending.pop(key, None)
                finished.append(key)
        return finished

    def idle(self) -> bool:
        return not self.pending

    def result(self, key: tuple) -> np.ndarray:
        t = self.trackers[key[0]]
        out = np.zeros(t.tally_size())
        t._ck(lib.mc_serve_result(t._h, key[1], C.c_void_p(out.ctypes.data), out.size), "mc_serve_result")
        return out

    def close(self) -> None:
        for t in self.trackers:
            lib.mc_serve_close(t._h)
            t.close()
        self.trackers = []


def poisson_jobs(problems: list[Problem], rate: float, duration: float, seed: int = 7,
                 hist_range=(1e4, 1e6)) -> list[Job]:
    """Arrivals at `rate` per second for `duration` seconds; each job picks a
    problem, a source point inside the middle half of its box, an energy
    from the Watt spectrum (a=0.988 MeV, b=2.249/MeV) and a log-uniform
    history count."""
    rng = np.random.default_rng(seed)
    jobs, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        k = int(rng.integers(len(problems)))
        p = problems[k]
        lo, hi = p.xyz.min(axis=0), p.xyz.max(axis=0)
        point = tuple(lo + (0.25 + 0.5 * rng.random(3)) * (hi - lo))
        while True:  # Watt: Maxwellian (T = a) plus shift
            w = -0.988e6 * (np.log(rng.random()) + np.log(rng.random()) * np.cos(np.pi / 2 * rng.random()) ** 2)
            e = w + 0.988e6 ** 2 * 2.249e-6 / 4 + (2 * rng.random() - 1) * np.sqrt(0.988e6 ** 2 * 2.249e-6 * w)
            if 1e-5 < e < 2e7:
                break
        n = int(np.exp(rng.uniform(np.log(hist_range[0]), np.log(hist_range[1]))))
        jobs.append(Job(k, n, int(rng.integers(1, 2**31)), point, float(e), t))
    return jobs


def run_stream(server: Server, jobs: list[Job]) -> dict:
    """Replays jobs at their arrival times; returns latency and throughput."""
    t0 = time.perf_counter()
    i, keys = 0, {}
    while i < len(jobs) or not server.idle():
        now = time.perf_counter() - t0
        while i < len(jobs) and jobs[i].arrival <= now:
            keys[server.submit(jobs[i])] = jobs[i]
            i += 1
        if server.idle():
            if i < len(jobs):
                time.sleep(max(0.0, min(0.002, jobs[i].arrival - now)))
            continue
        server.step()
    wall = time.perf_counter() - t0
    lat = np.array([server.done[k] - t0 - j.arrival for k, j in keys.items()])
    hist = sum(j.n_histories for j in jobs)
    return {"requests": len(jobs), "histories": hist, "wall_s": wall, "histories_per_s": hist / wall,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3)}


def run_one_at_a_time(trackers: list[Tracker], jobs: list[Job], precision: int = MC_PREC_FP64) -> dict:
    """Baseline: each request alone through mc_run, in arrival order."""
    t0 = time.perf_counter()
    lat = []
    for j in jobs:
        now = time.perf_counter() - t0
        if now < j.arrival:
            time.sleep(j.arrival - now)
        t = trackers[j.problem]
        t.set_source(Source(space=MC_SRC_POINT, energy=MC_SRC_MONO, point=j.point, mono_E=j.energy))
        t.run(j.n_histories, seed=j.seed, precision=precision, bank_size=min(j.n_histories, 1 << 20),
              accumulate=False)
        t.tally()  # result to the host
        t.reset_tally()
        lat.append(time.perf_counter() - t0 - j.arrival)
    wall = time.perf_counter() - t0
    lat = np.array(lat)
    hist = sum(j.n_histories for j in jobs)
    return {"requests": len(jobs), "histories": hist, "wall_s": wall, "histories_per_s": hist / wall,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3)}
