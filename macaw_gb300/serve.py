"""Serving form: a request loop over fixed-source problems.

A problem (mesh + cross sections) is made resident in its own context,
with its own CUDA stream, its particle bank and its request tally slots;
requests (problem, source point, energy, history count, seed) are queued
as they arrive, admitted by the C ABI's serving calls (mc_serve_*) into
free tally slots and run through that context's continuous event
pipeline, so requests on one problem share a particle bank and requests on
different problems overlap on separate streams.

Admission is by HBM footprint.  A problem's footprint is its resident
tables and bank plus its slots' tallies (footprint()); the problems
resident at once must fit the budget.  A request for a problem that is not
resident waits in the server's own queue until the problem can be made
resident: when it does not fit, problems with no request in flight are
evicted, least recently used first (their contexts closed, which frees
their device memory).  A problem is given as many slots (up to max_slots)
as the budget leaves room for, at least one.
"""
from __future__ import annotations

import ctypes as C
import time
from collections import deque
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


def footprint(p: Problem, bank: int, slots: int = 0) -> int:
    """Device bytes of a resident problem: mesh tables, cross sections,
    bank, and `slots` request tallies of one value per element (the default
    tally definition)."""
    return p.footprint_bytes() + bank * 250 + slots * p.n_tet * 8


class Server:
    def __init__(self, problems: list[Problem], device: int = 0, precision: int = MC_PREC_MIXED,
                 hbm_budget: int = 64 << 30, bank: int = 262144, max_seg: int = 64, max_slots: int = 8,
                 iterations: int = 4, preload: bool = True):
        self.problems = problems
        self.device, self.precision, self.bank, self.max_seg = device, precision, bank, max_seg
        self.max_slots, self.iterations, self.budget = max_slots, iterations, hbm_budget
        for p in problems:
            if footprint(p, bank, 1) > hbm_budget:
                raise MCError(1, f"problem {p.name} needs {footprint(p, bank, 1)} bytes with one slot, over the "
                                 f"HBM budget of {hbm_budget}")
        self.trackers: list[Tracker | None] = [None] * len(problems)
        self.slots: list[int] = [0] * len(problems)
        self.used: list[int] = [0] * len(problems)      # bytes each resident problem holds
        self.last_use: list[float] = [0.0] * len(problems)
        self.inflight: list[int] = [0] * len(problems)  # requests submitted to the context, not yet retired
        self.waiting: list[deque] = [deque() for _ in problems]  # requests whose problem is not resident yet
        self.loads = self.evictions = 0
        self.peak_bytes = 0
        self.pending: dict[tuple, float] = {}  # request key -> submit time
        self.done: dict[tuple, float] = {}     # request key -> completion time
        self._next_local = 0
        self._alias: dict[tuple, tuple] = {}   # (problem, ticket) -> request key, once submitted to the context
        self._unread: dict[tuple, tuple] = {}  # finished request key -> (problem, ticket), result not yet read
        self._saved: dict[tuple, np.ndarray] = {}  # results kept on the host when their problem was evicted
        if preload:
            # as many problems as fit, in order, each with an equal share of the spare room for slots
            share = hbm_budget // max(1, len(problems))
            for i, p in enumerate(problems):
                want = self._slots_for(p, share)
                if self.resident_bytes() + footprint(p, bank, want) <= hbm_budget:
                    self._load(i, want)

    # -- residency ----------------------------------------------------------
    def resident_bytes(self) -> int:
        return sum(self.used)

    def _slots_for(self, p: Problem, room: int) -> int:
        per = p.n_tet * 8
        base = footprint(p, self.bank, 0)
        return int(max(1, min(self.max_slots, (room - base) // per if room > base else 1)))

    def _load(self, i: int, n_slots: int) -> None:
        t = Tracker(self.device)
        t.load(self.problems[i])
        t._ck(lib.mc_serve_open(t._h, n_slots, self.bank, self.precision, self.max_seg), "mc_serve_open")
        self.trackers[i] = t
        self.slots[i] = n_slots
        self.used[i] = footprint(self.problems[i], self.bank, n_slots)
        self.loads += 1
        self.peak_bytes = max(self.peak_bytes, self.resident_bytes())

    def _evict(self, i: int) -> None:
        t = self.trackers[i]
        for key, (j, _) in list(self._unread.items()):
            if j == i:  # results not read yet outlive the context
                self._saved[key] = self.result(key)
        lib.mc_serve_close(t._h)
        t.close()
        self.trackers[i] = None
        self.slots[i] = 0
        self.used[i] = 0
        self.evictions += 1

    def _make_resident(self, i: int) -> bool:
        """Loads problem i, evicting idle problems (least recently used first)
        while it does not fit; False when it cannot fit yet."""
        p = self.problems[i]
        need = footprint(p, self.bank, 1)
        idle = sorted((j for j, t in enumerate(self.trackers) if t is not None and self.inflight[j] == 0),
                      key=lambda j: self.last_use[j])
        while self.resident_bytes() + need > self.budget and idle:
            self._evict(idle.pop(0))
        if self.resident_bytes() + need > self.budget:
            return False
        room = self.budget - self.resident_bytes()
        self._load(i, self._slots_for(p, room))
        return True

    # -- requests -----------------------------------------------------------
    def submit(self, job: Job) -> tuple:
        key = ("q", self._next_local)
        self._next_local += 1
        self.pending[key] = time.perf_counter()
        self.waiting[job.problem].append((key, job))
        self._admit(job.problem)
        return key

    def _admit(self, i: int) -> None:
        if not self.waiting[i]:
            return
        if self.trackers[i] is None and not self._make_resident(i):
            return
        t = self.trackers[i]
        while self.waiting[i]:
            key, job = self.waiting[i].popleft()
            r = Request()
            r.n_histories = job.n_histories
            r.seed = job.seed
            r.source.space = MC_SRC_POINT
            r.source.energy = MC_SRC_MONO
            r.source.point[:] = job.point
            r.source.mono_E = job.energy
            tk = C.c_int64()
            t._ck(lib.mc_serve_submit(t._h, C.byref(r), C.byref(tk)), "mc_serve_submit")
            self._alias[(i, tk.value)] = key
            self.inflight[i] += 1
        self.last_use[i] = time.perf_counter()

    def status(self, i: int) -> tuple[int, int, int]:
        """(queued, active, free slots) of resident problem i's context."""
        t = self.trackers[i]
        q, a, f = C.c_int32(), C.c_int32(), C.c_int32()
        t._ck(lib.mc_serve_status(t._h, C.byref(q), C.byref(a), C.byref(f)), "mc_serve_status")
        return q.value, a.value, f.value

    def step(self) -> list[tuple]:
        """Admit and launch on every resident problem, collect finished
        requests, then admit waiting requests whose problem can now be made
        resident."""
        busy = []
        for i, t in enumerate(self.trackers):
            if t is None or self.inflight[i] == 0:
                continue
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
                key = self._alias.pop((i, buf[k]))
                self.done[key] = now
                self.pending.pop(key, None)
                self._unread[key] = (i, buf[k])
                finished.append(key)
            self.inflight[i] -= n.value
            self.last_use[i] = now
        for i in range(len(self.problems)):
            self._admit(i)
        return finished

    def idle(self) -> bool:
        return not self.pending

    def result(self, key: tuple) -> np.ndarray:
        """FP64 tally of a finished request (raw sums per element); each
        result is read once."""
        if key in self._saved:
            return self._saved.pop(key)
        i, ticket = self._unread.pop(key)
        t = self.trackers[i]
        out = np.zeros(t.tally_size())
        t._ck(lib.mc_serve_result(t._h, ticket, C.c_void_p(out.ctypes.data), out.size), "mc_serve_result")
        return out

    def close(self) -> None:
        for i, t in enumerate(self.trackers):
            if t is not None:
                lib.mc_serve_close(t._h)
                t.close()
        self.trackers = [None] * len(self.problems)


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
    """Replays jobs at their arrival times; each finished request's tally is
    read back as it finishes (its latency ends there).  Returns latency,
    throughput and the server's residency record (loads, evictions, the
    most device bytes its resident problems held)."""
    t0 = time.perf_counter()
    i, keys, fin = 0, {}, {}
    while i < len(jobs) or not server.idle():
        now = time.perf_counter() - t0
        while i < len(jobs) and jobs[i].arrival <= now:
            keys[server.submit(jobs[i])] = jobs[i]
            i += 1
        if server.idle():
            if i < len(jobs):
                time.sleep(max(0.0, min(0.002, jobs[i].arrival - now)))
            continue
        for k in server.step():
            server.result(k)
            fin[k] = time.perf_counter()
    wall = time.perf_counter() - t0
    lat = np.array([fin[k] - t0 - j.arrival for k, j in keys.items()])
    hist = sum(j.n_histories for j in jobs)
    return {"requests": len(jobs), "histories": hist, "wall_s": wall, "histories_per_s": hist / wall,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "loads": server.loads, "evictions": server.evictions,
            "peak_resident_bytes": server.peak_bytes, "hbm_budget": server.budget}


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
