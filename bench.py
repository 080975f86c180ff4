#!/usr/bin/env python
"""Throughput of the particle-tracking hot path (histories/s).

Workload: the 17x17 pin-lattice fixed-source problem (2,039,184 tets, three
materials with 15/4/3 synthetic nuclides on 20,000-point grids, uniform
source in the fuel cylinders, Watt spectrum, vacuum boundary, FP64 element
track-length flux tally), tracked by the FP64 event-based GPU tracker in
batches ("steps") of 1,000,000 histories with a 1,000,000-particle bank.

  value  device-timed histories/s with inputs resident in HBM (source
         sampled on the device), CUDA events on the tracker's stream
  e2e    the same through the C ABI with host buffers: one pipelined
         mc_run streams the steps; each step's 1,000,000 source sites are
         copied from pinned host memory and each step's result (the SUM
         tally once its batch is folded in) is copied back to pinned host
         memory; "one_call_per_step" times one mc_run per step instead
  roofline  HBM roofline of the dominant kernel (the segment walk)
  cpu_baseline  the CPU restatement (oracle) on the host cores, bounded sample
  core, serve, eigen  the other forms at bounded sizes, each with its own
         clock record: the core at 1e7 histories in 64 batches (fixed
         parameters), a 5 s Poisson serving trace, two active k-eigenvalue
         generations of 1e6 (--no-extra leaves them out)

More workloads print their own JSON line (not the default run):
  --workload cube   the plain FP64 configuration the reference runs on CPU:
                    the 48,000-tet cube, 1e5 histories per step, FP64 and
                    mixed, with the oracle's segments and collisions per
                    history
  --workload core   the batched large-mesh form: cylindrical core, radius
                    180 cm, 400 cm, 41,283,792 tets, 200 materials of 5-40
                    nuclides (30,000-point grids); 1e8 histories in 64
                    batches of log-uniform size (1e5-5e6, rescaled) through
                    one pipelined, graph-replayed, autotuned call, and again
                    through one persistent launch, mixed and FP64 on the
                    same histories
  --workload eigen  the k-eigenvalue form: the lattice with fissionable fuel,
                    reflective sides (2,039,184 tets, k near 1); 1e6
                    particles per generation, W inactive then K active
                    generations per precision, fission-bank sort and
                    resampling on the device, keff of both precisions
  --workload serve  the serving form: a Poisson stream (50 requests/s) over
                    8 preloaded meshes of 10k-2M tets, continuous batching
                    with the mixed tracker and FP64 per-request tallies,
                    p50/p99 latency and throughput beside a one-request-at-
                    a-time FP64 loop on the same arrival trace

--impl reference times the reference path's CPU implementation (the oracle
restatement; MaCaw itself needs MOOSE/OpenMC/libMesh/MPI, absent here) on
the same workload; its inputs come from the oracle library's own build of
the generators, so that arm loads nothing of the CUDA tracker.
--profile-run runs one workload once, untimed, for ncu (run_profile).
Under torchrun every rank tracks its own history range (weak scaling, no
collective on the data path) and the ranks' SUM tallies are summed once
after the timed region (macaw_gb300/shard.py).
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "histories/s on 1 GB300, mixed vs plain FP64 at equal tally error; p50/p99 latency"
HIST_PER_STEP = 1_000_000
BANK = 1_000_000
B_SEG_FP64 = 164   # algorithmic bytes per segment: planes 128 + neighbours 16 + material 4 + tally RMW 16
B_SEG_MIXED = 84   # octahedral float planes 48 + neighbours 16 + material 4 + tally RMW 16
# per cross-section event: about 64 B per nuclide evaluated; an event on the
# lattice evaluates all three materials (15 + 4 + 3 nuclides); a collision
# re-reads 16 B per nuclide of its material to pick one (fuel: 15)
B_XS_EVENT = 64 * 22
B_COLL_PICK = 16 * 15
CPU_SAMPLE = 400_000
REF_SAMPLE = 100_000
# DRAM bytes per walked segment of the walk kernels, from ncu captures of
# every walk launch of a 2 x 2e5-history lattice run (profiles/walk_*_lattice.md);
# traffic per launch = this x the launch's segments
ADVANCE_DRAM_BYTES_PER_SEG = 181.0
MIXED_DRAM_BYTES_PER_SEG = 41.7
# what bounds each walk instead of HBM, from the same captures' --set full
# launch: the FP64 walk keeps the FP64 pipe 60% busy (GB300's FP64 rate is a
# 64th of its FP32 rate); the mixed walk waits on its one dependent record
# load per segment (L2 hit rate 48%, 29% of the warp slots occupied)
FP64_PIPE_ACTIVE = 0.597
MIXED_L2_HIT = 0.481
# the same captures' L2 hit rate and warp execution efficiency (active
# threads per executed instruction / 32), for the report
FP64_L2_HIT = 0.400
FP64_WARP_EFF = 23.37 / 32
MIXED_WARP_EFF = 20.30 / 32


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def workload_config():
    return {"workload": "lattice 17x17 pins, pitch 1.26 cm, 50 cm, 2,039,184 tets, 3 materials "
                        "(15/4/3 nuclides x 20,000 pts), cylinder source, 1e6 histories per step",
            "tets": 2039184, "histories_per_step": HIST_PER_STEP, "bank_size": BANK,
            "precision": "fp64", "mode": "event",
            "l2": "inputs larger than L2 (mesh planes 261 MB, tally 16 MB vs 129 MB L2)"}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons, sampled every 50 ms from before
    the warm-up on; stop(window) keeps the samples whose timestamps fall
    inside the timed region (wall-clock seconds from time.time())."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, window=None):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 10:
                    continue
                try:
                    ts = datetime.datetime.strptime(p[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                    rows.append((ts, float(p[2]), float(p[3]), [n for n, v in zip(names, p[6:10])
                                                                if v.lower() == "active"]))
                except ValueError:
                    continue
        os.unlink(self.path)
        inside = [r for r in rows if window and window[0] - 0.025 <= r[0] <= window[1] + 0.025]
        use = inside or rows
        sm = [r[1] for r in use]
        reasons = sorted({n for r in use for n in r[3]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(r[2] for r in use) if use else None,
                "reasons": reasons, "samples": len(sm), "in_timed_region": bool(inside)}


def history_roofline(hist_per_s, S, C, xs_evals, b_seg):
    """Whole-history algorithmic bytes (segments, cross-section lookups and
    collision nuclide picks) times histories/s against the HBM peak."""
    peak, _ = load_peaks()
    xs_events = xs_evals / 3.0  # each event evaluates the three materials
    b = S * b_seg + xs_events * B_XS_EVENT + C * B_COLL_PICK
    return {"bytes_per_history": b, "achieved": hist_per_s * b / 1e9, "unit": "GB/s", "peak": peak,
            "frac": hist_per_s * b / 1e9 / peak,
            "formula": "S*B_seg + xs_events*64*22 + C*16*15 (S, C, xs events per history measured)"}


def cpu_baseline(problem, sample, seed=1):
    from oracle.oracle import Oracle, cpu_threads
    threads = cpu_threads()
    o = Oracle(problem)
    o.run(2000, first=10**9, seed=seed, threads=threads, traces=False)  # warm caches, page in
    _, _, st, dt = o.run(sample, first=0, seed=seed, threads=threads, traces=False)
    one = max(2000, sample // 20)
    _, _, _, dt1 = o.run(one, first=sample, seed=seed, threads=1, traces=False)
    return {"value": sample / dt, "unit": "histories/s", "cores": threads, "kind": "port",
            "sample": f"{sample} histories of the same lattice workload (C oracle, OpenMP over histories)",
            "seconds": dt, "segments_per_history": st["n_seg"] / sample,
            "collisions_per_history": st["n_coll"] / sample,
            "single_core": {"value": one / dt1, "sample": f"{one} histories on one thread"}}


def run_reference(args):
    rank = env_int("RANK", 0)
    if rank != 0:
        return 0
    # the inputs come from the oracle library's own build of the generator
    # sources: this arm loads no part of the CUDA tracker
    from macaw_gb300 import problems
    from oracle.oracle import Oracle, cpu_threads, generator_library
    problems.use_generator_library(generator_library())
    p = problems.lattice_problem()
    threads = cpu_threads()
    o = Oracle(p)
    n = REF_SAMPLE
    for w in range(args.warmup):
        o.run(n, first=w * n, seed=1, threads=threads, traces=False)
    t0 = time.perf_counter()
    segs = 0
    for k in range(args.steps):
        _, _, st, _ = o.run(n, first=(args.warmup + k) * n, seed=1, threads=threads, traces=False)
        segs += st["n_seg"]
    dt = time.perf_counter() - t0
    v = n * args.steps / dt
    cfg = workload_config()
    cfg["histories_per_step"] = n
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "histories/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generators; the reference's meshes and ENDF data are not shipped)",
            "config": cfg, "segments_per_s": segs / dt,
            "cpu_baseline": {"value": v, "unit": "histories/s", "cores": threads, "kind": "port",
                             "sample": f"{n} histories per step of the lattice workload; the reference "
                                       "(MOOSE+OpenMC) cannot be built, the oracle restates its CPU path"},
            "e2e": {"value": v, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def core_batch_sizes(total=100_000_000, n=64, lo=1e5, hi=5e6, seed=64):
    import numpy as np
    rng = np.random.default_rng(seed)
    s = np.exp(rng.uniform(np.log(lo), np.log(hi), n))
    s = np.floor(s * (total / s.sum())).astype(np.int64)
    s[-1] += total - s.sum()
    return s


def core_result(total, tune=True, batches=64):
    """Batched large-mesh form: mixed and FP64 on the same histories, each
    leg through one pipelined call of log-uniform batches, with its own
    clock record.  tune: the autotuner picks each leg's parameters (else the
    parameters it picked on this workload before)."""
    import numpy as np
    import torch
    from macaw_gb300 import Tracker, problems
    from macaw_gb300._lib import MC_PREC_FP64, MC_PREC_MIXED, MC_TALLY_SUM
    from macaw_gb300.tracker import run_persistent
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    p = problems.core_problem()
    sizes = core_batch_sizes(total, n=batches)
    stream = torch.cuda.Stream()
    # particles in flight: the mixed walk gains from a larger bank on this
    # mesh (more particles per element bucket of the ordered queue; 10.1M ->
    # 11.2M histories/s from 2M to 8M), the FP64 walk does not
    banks = {"mixed": 8_000_000, "fp64": 2_000_000}
    fixed = {"mixed": {"block_size": 256, "max_seg": 128, "sort_queue": 13, "refill": False, "graph": True},
             "fp64": {"block_size": 256, "max_seg": 64, "sort_queue": 13, "refill": False, "graph": True,
                      "walk_blocks": 4}}
    out = {"metric": "histories/s, batched large-mesh form", "unit": "histories/s", "n_gpus": 1,
           "higher_is_better": True, "dtype": "f32+f64",
           "data": "synthetic (seeded generators)",
           "config": {"workload": f"core R=180 cm H=400 cm, {p.n_tet} tets, 200 materials x 5-40 nuclides x "
                                  f"30,000 pts; {int(sizes.sum())} histories in {sizes.size} batches "
                                  f"({int(sizes.min())}..{int(sizes.max())})", "tets": p.n_tet,
                      "histories": int(sizes.sum()), "bank_size": banks,
                      "l2": "inputs larger than L2 (mesh tables about 10 GB)"}}
    res = {}
    t = Tracker(0)
    t.load(p)
    t.set_stream(stream.cuda_stream)
    for name, prec in (("mixed", MC_PREC_MIXED), ("fp64", MC_PREC_FP64)):
        if tune:
            params, _ = t.autotune(trial=1_000_000, first=10**10, bank_size=banks[name], precision=prec,
                                   block_size=256, max_seg=64)
            params["graph"] = True if name == "mixed" else params["graph"]
        else:
            params = dict(fixed[name], bank_size=banks[name])
        t.reset_tally()
        t.run(int(sizes[:3].sum()), first=2 * 10**10, seed=1, precision=prec, accumulate=True,
              batch_sizes=sizes[:3], **params)  # warm-up
        if name == "mixed":
            out["setup_s"] = time.perf_counter() - t0
        t.reset_tally()
        torch.cuda.synchronize()
        clk = ClockSampler(0)
        clk.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0 = time.time()
        e0.record(stream)
        st = t.run(int(sizes.sum()), first=0, seed=1, precision=prec, accumulate=True, batch_sizes=sizes,
                   **params)
        e1.record(stream)
        torch.cuda.synchronize()
        clocks = clk.stop((c0, time.time()))
        ms = e0.elapsed_time(e1)
        res[name] = {"value": int(sizes.sum()) / (ms / 1e3), "ms": ms, "tuned": params,
                     "segments_per_s": st.n_seg / (ms / 1e3), "segments_per_history": st.n_seg / sizes.sum(),
                     "xs_per_history": st.n_xs / sizes.sum(), "stuck": int(st.n_stuck), "lost": int(st.n_lost),
                     "fallback_fraction": st.n_fallback / max(st.n_seg, 1), "gpu_launches": int(st.n_launch),
                     "batches_done": t.batches_done(), "clocks": clocks}
        res[name]["sum"] = t.tally(MC_TALLY_SUM)
        # the same batches as one persistent launch (one tally slot per batch)
        firsts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
        t.reset_tally()
        clk = ClockSampler(0)
        clk.start()
        c0 = time.time()
        pst, _ = run_persistent([(t, int(f), int(n), 1) for f, n in zip(firsts, sizes)], precision=prec)
        res[name]["persistent"] = {"value": int(sizes.sum()) / (pst.ms_total / 1e3), "ms": pst.ms_total,
                                   "segments_per_history": pst.n_seg / sizes.sum(), "stuck": int(pst.n_stuck),
                                   "lost": int(pst.n_lost), "gpu_launches": int(pst.n_launch),
                                   "batches_done": t.batches_done(), "clocks": clk.stop((c0, time.time()))}
    t.close()
    a, b = res["mixed"].pop("sum"), res["fp64"].pop("sum")
    nz = b > 0
    rel = np.abs(a[nz] - b[nz]) / b[nz]
    blk = p.tet_block
    fb = np.bincount(blk, weights=b)
    mb = np.bincount(blk, weights=a)
    okb = fb > 0
    relb = np.abs(mb[okb] - fb[okb]) / fb[okb]
    out.update({"value": res["mixed"]["value"], "mixed": res["mixed"], "fp64": res["fp64"],
                "speedup_vs_fp64": res["mixed"]["value"] / res["fp64"]["value"],
                "flux_rel_diff_mean": float(rel.mean()), "flux_rel_diff_max": float(rel.max()),
                "flux_rel_diff_block_max": float(relb.max()),
                "flux_rel_diff_note": "SUM tallies, mixed vs FP64 on the same histories: per element with a score "
                                      "(mean, max) and per block (material region, max)",
                "forms_note": "each leg: the batches through one pipelined, graph-replayed mc_run (value) and "
                              "through one persistent launch, mc_run_persistent (persistent)"})
    return out


def run_core(args):
    """Batched large-mesh form (one JSON line)."""
    print(json.dumps(core_result(args.core_histories, tune=not args.no_tune)))
    return 0


def run_cube(args):
    """The plain FP64 configuration the reference runs on CPU: the 48,000-tet
    cube, 1e5 histories per step (one JSON line); S and C from the oracle."""
    import torch
    from macaw_gb300 import Tracker, problems
    from macaw_gb300._lib import MC_PREC_FP64, MC_PREC_MIXED
    from oracle.oracle import Oracle, cpu_threads
    torch.cuda.set_device(0)
    p = problems.cube_problem()
    n, K = 100_000, max(args.steps, 1)
    o = Oracle(p)
    threads = cpu_threads()
    _, _, ost, odt = o.run(n, first=0, seed=1, threads=threads, traces=False)
    res = {}
    with Tracker(0) as t:
        t.load(p)
        for name, prec in (("fp64", MC_PREC_FP64), ("mixed", MC_PREC_MIXED)):
            kw = dict(seed=1, precision=prec, accumulate=True, bank_size=n, max_seg=64, sort_queue=0, graph=True)
            t.run(n * 3, first=10**8, batch_sizes=[n] * 3, **kw)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            st = t.run(n * K, first=0, batch_sizes=[n] * K, **kw)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            res[name] = {"value": n * K / (ms / 1e3), "ms_per_step": ms / K, "segments_per_history": st.n_seg / (n * K),
                         "collisions_per_history": st.n_coll / (n * K), "stuck": int(st.n_stuck), "lost": int(st.n_lost)}
    out = {"metric": "histories/s, plain FP64 cube configuration", "unit": "histories/s", "n_gpus": 1,
           "value": res["fp64"]["value"], "higher_is_better": True, "dtype": "f64", "steps": K,
           "data": "synthetic (seeded generators)",
           "config": {"workload": "cube 20 cm, 20^3 hexes x 6 tets (48,000 tets), 1 material x 10 nuclides x "
                                  "10,000 pts, point source at the centre, 1e5 histories per step", "tets": p.n_tet},
           "fp64": res["fp64"], "mixed": res["mixed"],
           "oracle": {"segments_per_history": ost["n_seg"] / n, "collisions_per_history": ost["n_coll"] / n,
                      "histories_per_s": n / odt, "cores": threads}}
    print(json.dumps(out))
    return 0


def eigen_result(n, K, W, no_mixed=False, cpu=True):
    """k-eigenvalue form (one JSON line): generations of 1e6 particles on the
    fissionable lattice; value = active-generation histories / device time
    of those generations (tracking, estimator sums, bank sort and
    resampling; CUDA events on the tracker's stream)."""
    import numpy as np
    import torch
    from macaw_gb300 import Tracker, problems
    from macaw_gb300._lib import MC_PREC_FP64, MC_PREC_MIXED
    from oracle.oracle import Oracle, cpu_threads
    torch.cuda.set_device(0)
    p = problems.eigen_lattice_problem()
    res = {}
    with Tracker(0) as t:
        t.load(p)
        # walk budget and block from a sweep on this workload (8-32 segments,
        # 128/256 threads): flights here are about 28 segments long
        for name, prec, ms_ in (("fp64", MC_PREC_FP64, 32), ("mixed", MC_PREC_MIXED, 32)):
            if name == "mixed" and no_mixed:
                continue
            clk = ClockSampler(0)
            clk.start()
            w0 = time.perf_counter()
            c0 = time.time()
            g = t.eigen(n, W + K, W, seed=1, precision=prec, bank_size=n, max_seg=ms_, sort_queue=9, graph=True,
                        block_size=128)
            wall = time.perf_counter() - w0
            clocks = clk.stop((c0, time.time()))
            act = g[W:]
            ms = float(act["ms"].sum())
            S = float(act["n_seg"].sum()) / (n * K)
            Cc = float(act["n_coll"].sum()) / (n * K)
            res[name] = {"value": n * K / (ms / 1e3), "ms_per_generation": ms / K,
                         "wall_histories_per_s": n * (W + K) / wall,
                         "keff": float(act["keff"][-1]), "keff_std": float(act["keff_std"][-1]),
                         "k_collision_mean": float(act["k_collision"].mean()),
                         "k_absorption_mean": float(act["k_absorption"].mean()),
                         "sites_per_generation": float(act["n_sites"].mean()),
                         "segments_per_history": S, "collisions_per_history": Cc,
                         "leakage": float(act["leakage"].mean()), "clocks": clocks}
    peak, psrc = load_peaks()
    f = res["fp64"]
    # algorithmic bytes per history: segments (FP64 records, tally RMW), one
    # cross-section event per flight (22 nuclides), a pick per collision, and
    # per banked site its write, the sort's read and write and the
    # resampled source write (80 + 160 + 64 B)
    sites_ph = f["sites_per_generation"] / n
    b_h = f["segments_per_history"] * B_SEG_FP64 + (f["collisions_per_history"] + 1) * B_XS_EVENT + \
        f["collisions_per_history"] * B_COLL_PICK + sites_ph * (80 + 160 + 64)
    out = {"metric": "histories/s, k-eigenvalue generations", "unit": "histories/s", "n_gpus": 1,
           "value": f["value"], "higher_is_better": True, "dtype": "f64", "steps": K, "warmup": W,
           "data": "synthetic (seeded generators)",
           "config": {"workload": f"eigen lattice 17x17 pins, 50 cm, {p.n_tet} tets, every fuel nuclide "
                                  f"fissionable, reflective sides, vacuum top/bottom; {n} particles per generation, "
                                  f"{W} inactive + {K} active generations", "tets": p.n_tet,
                      "l2": "inputs larger than L2 (mesh planes 261 MB, bank 80 MB)"},
           "fp64": f, "mixed": res.get("mixed"),
           "speedup_mixed_vs_fp64": res["mixed"]["value"] / f["value"] if "mixed" in res else None,
           "roofline_history": {"bytes_per_history": b_h, "achieved": f["value"] * b_h / 1e9, "unit": "GB/s",
                                "peak": peak, "peak_source": psrc, "frac": f["value"] * b_h / 1e9 / peak,
                                "formula": "S*164 + (C+1)*64*22 + C*16*15 + sites*(80+160+64), FP64"}}
    if cpu:
        threads = cpu_threads()
        o = Oracle(p)
        n_cpu = 20_000
        og, _, _, _, odt = o.eigen(n_cpu, 2, 1, seed=1, threads=threads)
        out["cpu_baseline"] = {"value": n_cpu * 2 / odt, "unit": "histories/s", "cores": threads, "kind": "port",
                               "sample": f"{n_cpu} particles x 2 generations of the same problem (C oracle)",
                               "keff_generation": [float(x) for x in og["k_generation"]]}
    return out


def run_eigen(args):
    """k-eigenvalue form (one JSON line)."""
    print(json.dumps(eigen_result(1_000_000, max(args.steps, 1), args.warmup, args.no_mixed)))
    return 0


def serve_problems():
    from macaw_gb300 import problems
    cubes = [(12, 12.0), (20, 20.0), (40, 40.0), (60, 60.0)]
    lats = [(5, 5, 10, 20.0), (9, 9, 15, 30.0), (13, 13, 20, 40.0), (17, 17, 21, 50.0)]
    ps = [problems.cube_problem(n=n, L=L, seed=1000 + i) for i, (n, L) in enumerate(cubes)]
    ps += [problems.lattice_problem(nx=a, ny=b, nz=c, height=h, seed=2000 + i) for i, (a, b, c, h) in enumerate(lats)]
    return ps


def serve_result(seconds):
    """Serving form: a seeded Poisson trace (50 requests/s for `seconds` s)
    through the continuous-batching server (mixed tracker), then the same
    trace one request at a time in FP64; each with its own clock record."""
    import torch
    from macaw_gb300 import Tracker
    from macaw_gb300._lib import MC_PREC_FP64, MC_PREC_MIXED
    from macaw_gb300.serve import Server, poisson_jobs, run_one_at_a_time, run_stream
    torch.cuda.set_device(0)
    ps = serve_problems()
    jobs = poisson_jobs(ps, rate=50.0, duration=seconds, seed=7, hist_range=(1e4, 1e6))
    srv = Server(ps, precision=MC_PREC_MIXED, hbm_budget=96 << 30, bank=1 << 20, max_slots=8)
    warm = poisson_jobs(ps, rate=50.0, duration=1.0, seed=8, hist_range=(1e4, 1e5))
    run_stream(srv, warm)
    clk = ClockSampler(0)
    clk.start()
    c0 = time.time()
    rep = run_stream(srv, jobs)
    rep["clocks"] = clk.stop((c0, time.time()))
    slots = list(srv.slots)
    srv.close()
    trackers = [Tracker(0).load(p) for p in ps]
    run_one_at_a_time(trackers, warm[:8], precision=MC_PREC_FP64)
    clk = ClockSampler(0)
    clk.start()
    c0 = time.time()
    base = run_one_at_a_time(trackers, jobs, precision=MC_PREC_FP64)
    base["clocks"] = clk.stop((c0, time.time()))
    for t in trackers:
        t.close()
    out = {"metric": "serving: histories/s and p50/p99 request latency", "unit": "histories/s",
           "value": rep["histories_per_s"], "n_gpus": 1, "higher_is_better": True, "dtype": "f32+f64",
           "data": "synthetic (seeded generators and arrival trace)",
           "config": {"workload": f"Poisson 50 requests/s for {seconds} s over 8 meshes "
                                  f"({', '.join(str(p.n_tet) for p in ps)} tets), point sources, Watt energies, "
                                  "log-uniform 1e4..1e6 histories", "slots_per_mesh": slots,
                      "requests": rep["requests"], "histories": rep["histories"]},
           "serving": rep, "one_at_a_time_fp64": base,
           "p50_speedup": base["p50_ms"] / rep["p50_ms"], "p99_speedup": base["p99_ms"] / rep["p99_ms"]}
    return out


def run_serve(args):
    """Serving form (one JSON line)."""
    print(json.dumps(serve_result(args.serve_seconds)))
    return 0


def run_profile(args):
    """Runs one workload once for a profiler (ncu), no timing: one untimed
    batch (so every kernel's first launch is warm), then `--batches` batches
    of `--hist` histories through one pipelined call with fixed parameters
    (the autotuner's choices on the workload unless overridden); prints the
    run's statistics as JSON.  --workload eigen: one inactive generation,
    then `--batches` active ones of `--hist` particles in one call.

      python bench.py --profile-run --workload lattice --precision fp64 --hist 200000 --batches 1
    """
    from macaw_gb300 import Tracker, problems
    from macaw_gb300._lib import MC_PREC_FP64, MC_PREC_MIXED
    prec = MC_PREC_MIXED if args.precision == "mixed" else MC_PREC_FP64
    block = args.block or (64 if prec == MC_PREC_MIXED else 128)
    max_seg = args.max_seg or (128 if prec == MC_PREC_MIXED else 64)
    sort = args.sort or (13 if args.workload == "core" else 9)
    n = args.hist
    if args.workload == "eigen":
        p = problems.eigen_lattice_problem(nx=args.pins, ny=args.pins)
        with Tracker(0) as t:
            t.load(p)
            g = t.eigen(n, 1 + args.batches, 1, seed=1, precision=prec, bank_size=n, block_size=block,
                        max_seg=max_seg, sort_queue=sort, graph=True)
            print(json.dumps([{k: g[k][i].item() for k in g.dtype.names} for i in range(g.size)]))
        return 0
    if args.workload not in ("lattice", "core"):
        raise SystemExit("--profile-run takes --workload lattice, core or eigen")
    p = problems.lattice_problem(nx=args.pins, ny=args.pins) if args.workload == "lattice" \
        else problems.core_problem(pins=args.pins, radius=args.radius)
    with Tracker(0) as t:
        t.load(p)
        kw = dict(bank_size=n, block_size=block, max_seg=max_seg, sort_queue=sort, precision=prec,
                  walk_blocks=args.walk_blocks)
        warm = t.run(n, first=0, seed=1, accumulate=True, **kw).as_dict()
        st = t.run(n * args.batches, first=n, seed=1, accumulate=True, batch_sizes=[n] * args.batches, **kw)
        print(json.dumps(dict(st.as_dict(), warm=warm)))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (fixed parameters)")
    ap.add_argument("--hist", type=int, default=HIST_PER_STEP)
    ap.add_argument("--workload", default="lattice", choices=["lattice", "cube", "core", "serve", "eigen"])
    ap.add_argument("--core-histories", type=int, default=100_000_000)
    ap.add_argument("--serve-seconds", type=float, default=20.0)
    ap.add_argument("--no-extra", action="store_true",
                    help="default run: leave out the core, serve and eigen sub-objects")
    ap.add_argument("--profile-run", action="store_true",
                    help="run one workload once with fixed parameters for a profiler (ncu); see run_profile")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64", help="--profile-run only")
    ap.add_argument("--batches", type=int, default=2, help="--profile-run only")
    ap.add_argument("--pins", type=int, default=17, help="--profile-run only: pin cells per lattice side")
    ap.add_argument("--block", type=int, default=0, help="--profile-run only")
    ap.add_argument("--max-seg", type=int, default=0, help="--profile-run only: 0 = 128 mixed, 64 fp64")
    ap.add_argument("--sort", type=int, default=0, help="--profile-run only: 0 = 9 (lattice), 13 (core)")
    ap.add_argument("--radius", type=float, default=180.0, help="--profile-run only: core radius (cm)")
    ap.add_argument("--walk-blocks", type=int, default=0,
                    help="--profile-run only: FP64 walk build, 4 or 5 resident blocks per SM (0 = 5)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.profile_run:
        return run_profile(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "core":
        return run_core(args)
    if args.workload == "cube":
        return run_cube(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "eigen":
        return run_eigen(args)

    import numpy as np
    import torch

    rank, world, local = env_int("RANK", 0), env_int("WORLD_SIZE", 1), env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from macaw_gb300 import Tracker, problems
    from macaw_gb300._lib import MC_PREC_FP64, MC_PREC_MIXED, MC_TALLY_SUM, SITE_DTYPE

    n, K, W = args.hist, args.steps, args.warmup
    p = problems.lattice_problem()
    stream = torch.cuda.Stream()
    # each rank owns a disjoint range of history indices (weak scaling)
    base = rank * (W + 2 * K + 5) * n

    def barrier():
        if dist is not None:
            dist.barrier()

    def tracker():
        t = Tracker(local)
        t.load(p)
        t.set_stream(stream.cuda_stream)
        return t

    def tune(t, precision):
        fixed = {"bank_size": BANK, "block_size": 128, "max_seg": 64 if precision == MC_PREC_FP64 else 128,
                 "sort_queue": 9, "refill": False, "graph": True}
        if args.no_tune:
            return fixed, None
        # trials: four pipelined batches of n histories, the batch size of
        # the timed steps (with batches of n/2 the tuner picked a mixed walk
        # budget 3% slower on the steps)
        params, rate = t.autotune(trial=4 * n, first=base + (W + 2 * K + 1) * n, bank_size=BANK,
                                  precision=precision, block_size=128, max_seg=64, sort_queue=9)
        return params, rate

    def timed(t, precision, params, first_step, steps, profile):
        """steps batches of n histories through one pipelined call; device ms."""
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = t.run(n * steps, first=base + first_step * n, seed=1, precision=precision, accumulate=True,
                   batch_sizes=[n] * steps, profile=profile, **params)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1)
        if dist is not None:
            tt = torch.tensor([ms], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            ms = float(tt.item())
        return ms, st

    # --- FP64 (the configuration the metric is quoted on) ---
    t = tracker()
    params64, tune64 = tune(t, MC_PREC_FP64)
    clocks = ClockSampler(local)
    clocks.start()
    timed(t, MC_PREC_FP64, params64, 0, W, False)
    w0 = time.time()
    ms, st = timed(t, MC_PREC_FP64, params64, W, K, False)
    clk = clocks.stop((w0, time.time()))
    value = world * n * K / (ms / 1e3)
    sum64 = t.tally(MC_TALLY_SUM)
    reduce_ms = None
    if dist is not None:
        # the one exchange step of a sharded run: an FP64 sum of the element
        # tallies over the ranks (after the timed region)
        from macaw_gb300.shard import reduce_tally
        r0 = time.perf_counter()
        sum64 = reduce_tally(sum64)
        reduce_ms = (time.perf_counter() - r0) * 1e3
    # the K steps once more on the next histories, pipelined as in the timed
    # region, with the walk launches timed (CUDA events around each walk
    # launch, which turns graph replay off), for the walk's roofline: a
    # single batch would time the walk while its queue drains, which is not
    # the state the timed steps run in
    _, pst64 = timed(t, MC_PREC_FP64, params64, W + K, K, True)

    # --- mixed-precision form on the same histories ---
    mixed = None
    if not args.no_mixed:
        tm = tracker()
        paramsm, tunem = tune(tm, MC_PREC_MIXED)
        clocks_m = ClockSampler(local)
        clocks_m.start()
        timed(tm, MC_PREC_MIXED, paramsm, 0, W, False)
        w0m = time.time()
        mms, mst = timed(tm, MC_PREC_MIXED, paramsm, W, K, False)
        clk_m = clocks_m.stop((w0m, time.time()))
        summ = tm.tally(MC_TALLY_SUM)
        # the K steps once more with the walk launches timed, for the walk's roofline
        _, pst = timed(tm, MC_PREC_MIXED, paramsm, W + K, K, True)
        nz = sum64 > 0
        rel = np.abs(summ[nz] - sum64[nz]) / sum64[nz]
        mixed = {"value": world * n * K / (mms / 1e3), "unit": "histories/s", "ms_per_step": mms / K,
                 "speedup_vs_fp64": ms / mms, "fallback_fraction": mst.n_fallback / max(mst.n_seg, 1),
                 "stuck": int(mst.n_stuck), "lost": int(mst.n_lost),
                 "flux_rel_diff_mean": float(rel.mean()), "flux_rel_diff_max": float(rel.max()),
                 "flux_rel_diff_note": "element SUM tallies, mixed vs FP64 (bit-exact to the oracle), same "
                                       f"{n * (W + K)} histories, elements with a score",
                 "tuned": paramsm, "gpu_launches": int(mst.n_launch), "clocks": clk_m,
                 "roofline_history": history_roofline(world * n * K / (mms / 1e3), mst.n_seg / (n * K),
                                                      mst.n_coll / (n * K), mst.n_xs / (n * K), B_SEG_MIXED)}
        if pst.ms_advance > 0:
            mach = pst.n_seg_advance * B_SEG_MIXED / (pst.ms_advance / 1e3) / 1e9
            mixed["roofline"] = {"bound": "hbm", "kernel": "k_ev_advance<MIXED>" if paramsm.get("refill")
                                 else "k_ev_advance_mixed", "achieved": mach, "unit": "GB/s",
                                 "algorithmic_bytes_per_segment": B_SEG_MIXED,
                                 "advance_ms_per_launch": pst.ms_advance / max(pst.n_advance_launch, 1),
                                 "segments_per_launch": pst.n_seg_advance / max(pst.n_advance_launch, 1),
                                 "traffic": MIXED_DRAM_BYTES_PER_SEG * pst.n_seg_advance / max(pst.n_advance_launch, 1),
                                 "limiter": {"dependent_record_loads_l2_hit": MIXED_L2_HIT,
                                             "source": "ncu lts__t_sector_hit_rate (profiles/walk_mixed_lattice.md)"},
                                 "l2_hit_rate": MIXED_L2_HIT, "warp_execution_efficiency": MIXED_WARP_EFF,
                                 "sample": f"{K} more batches of {n} histories pipelined as in the timed region, "
                                           "each walk launch timed by CUDA events (graph replay off)"}

    # --- end to end through the C ABI with host buffers ---
    # One pipelined mc_run streams the K steps: every step's 1e6 source sites
    # are copied in from pinned host memory, and every step's result (the
    # SUM tally as it stands once that step's batch is folded in) is copied
    # out to its own pinned host buffer while later steps run.
    k0 = W + K
    site_buf = torch.empty(K * n * SITE_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
    site_np = site_buf.numpy().view(SITE_DTYPE)
    t.sample_sites(K * n, first=base + k0 * n, seed=1, out=site_np)
    outs = [torch.empty(p.n_tet, dtype=torch.float64).pin_memory() for _ in range(K)]
    outs_np = [o.numpy() for o in outs]

    def e2e_run(tr, precision, params):
        barrier()
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        tr.run(K * n, first=base + k0 * n, seed=1, precision=precision, accumulate=True, sites=site_np,
               batch_sizes=[n] * K, batch_results=outs_np, **params)
        torch.cuda.synchronize()
        barrier()
        sec = time.perf_counter() - w0
        if dist is not None:
            tt = torch.tensor([sec], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            sec = float(tt.item())
        return sec

    def e2e_per_call(tr, precision, params):
        """The same steps as one mc_run per step (each with its own tail)."""
        barrier()
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        for k in range(K):
            tr.run(n, first=base + (k0 + k) * n, seed=1, precision=precision, accumulate=True,
                   sites=site_np[k * n:(k + 1) * n], **params)
            tr.tally(MC_TALLY_SUM, out=outs_np[k])
        torch.cuda.synchronize()
        barrier()
        return time.perf_counter() - w0

    e2e_s = e2e_run(t, MC_PREC_FP64, params64)
    e2e_call_s = e2e_per_call(t, MC_PREC_FP64, params64)
    if mixed is not None:
        m_s = e2e_run(tm, MC_PREC_MIXED, paramsm)
        m_call_s = e2e_per_call(tm, MC_PREC_MIXED, paramsm)
        mixed["e2e"] = {"value": world * n * K / m_s, "unit": "histories/s",
                        "h2d_bytes_per_step": n * SITE_DTYPE.itemsize, "d2h_bytes_per_step": p.n_tet * 8,
                        "one_call_per_step": world * n * K / m_call_s}
        tm.close()
    e2e = {"value": world * n * K / e2e_s, "unit": "histories/s",
           "h2d_bytes_per_step": n * SITE_DTYPE.itemsize, "d2h_bytes_per_step": p.n_tet * 8,
           "note": "one pipelined mc_run for the K steps: each step's 1e6 host sites copied in (pinned), each "
                   "step's SUM tally copied out to pinned host memory as its batch folds; the host sites are "
                   "sampled on the device before the timed region, so source sampling is outside this clock "
                   "(it is inside the device-timed value)",
           "one_call_per_step": world * n * K / e2e_call_s}

    if rank == 0:
        peak, peak_kind = load_peaks()
        segs = st.n_seg
        walk = pst64.n_seg_advance  # segments inside the timed walk launches (the rest: tail kernel)
        adv_bytes = walk * B_SEG_FP64
        achieved = adv_bytes / (pst64.ms_advance / 1e3) / 1e9 if pst64.ms_advance > 0 else None
        roof = {"bound": "hbm", "kernel": "k_ev_advance<FP64>" if params64.get("refill")
                else "k_ev_advance_fp64",
                "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None,
                "traffic": (ADVANCE_DRAM_BYTES_PER_SEG * walk / max(pst64.n_advance_launch, 1))
                if ADVANCE_DRAM_BYTES_PER_SEG else None,
                "segments_per_launch": walk / max(pst64.n_advance_launch, 1),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "algorithmic_bytes_per_segment": B_SEG_FP64,
                "advance_ms_per_launch": pst64.ms_advance / max(pst64.n_advance_launch, 1),
                "advance_share_of_step": pst64.ms_advance / pst64.ms_total if pst64.ms_total > 0 else None,
                "sample": f"{K} more batches of {n} histories pipelined as in the timed region, each walk launch "
                          "timed by CUDA events (graph replay off)",
                "traffic_source": "ncu DRAM bytes per walked segment (profiles/walk_fp64_lattice.md) x segments "
                                  "per launch",
                "limiter": {"fp64_pipe_active": FP64_PIPE_ACTIVE,
                            "source": "ncu sm__pipe_fp64_cycles_active (profiles/walk_fp64_lattice.md)"},
                "l2_hit_rate": FP64_L2_HIT, "warp_execution_efficiency": FP64_WARP_EFF,
                "counters_source": "ncu lts__t_sector_hit_rate and smsp__thread_inst_executed_per_inst_executed "
                                   "(profiles/walk_*_lattice.md)",
                "note": "the FP64 walk is bound by GB300's FP64 pipe, not HBM (see profiles/)"}
        cfg = dict(workload_config(), parallelism=f"replicas{world}" if world > 1 else "single",
                   pipelined_batches=K, tuned=params64)
        if mixed is not None and "roofline" in mixed:
            mixed["roofline"]["peak"] = peak
            mixed["roofline"]["frac"] = mixed["roofline"]["achieved"] / peak
        line = {"metric": METRIC, "value": value, "unit": "histories/s", "n_gpus": world, "steps": K,
                "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generators; the reference's meshes and ENDF data are not shipped)",
                "config": cfg, "segments_per_s": world * segs / (ms / 1e3), "segments_per_history": segs / (n * K),
                "collisions_per_history": st.n_coll / (n * K),
                "roofline_history": history_roofline(value, segs / (n * K), st.n_coll / (n * K),
                                                     st.n_xs / (n * K), B_SEG_FP64),
                "stuck": int(st.n_stuck), "lost": int(st.n_lost),
                "roofline": roof, "e2e": e2e, "gpu_launches": int(st.n_launch), "clocks": clk}
        if reduce_ms is not None:
            line["tally_reduce_ms"] = reduce_ms
        if mixed is not None:
            line["mixed"] = mixed
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(p, CPU_SAMPLE)
    t.close()
    if rank == 0:
        if world == 1 and not args.no_extra:
            # the other forms, bounded so the default run stays within minutes
            # (each sub-object carries its own clock record; the workload
            # names state its size)
            extra = {}
            for key, fn in (("core", lambda: core_result(10_000_000, tune=False)),
                            ("serve", lambda: serve_result(5.0)),
                            ("eigen", lambda: eigen_result(1_000_000, 2, 1, cpu=False))):
                try:
                    extra[key] = fn()
                except Exception as e:  # reported, never silently dropped
                    extra[key] = {"error": f"{type(e).__name__}: {e}"}
            line.update(extra)
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
