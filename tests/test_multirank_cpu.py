"""Multi-rank sharding of histories (world_size 2, gloo, CPU).

Across GPUs the path shards by history index: rank r tracks a disjoint
range of particle ids, and the only exchange is one FP64 sum-reduce of the
element tallies at the end.  Because every history's random numbers are
keyed by its global id, the sharded result must equal a single-rank run:
per-history traces identical, tallies equal up to summation order.  The
ranks here run the oracle on the CPU and reduce over gloo.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

N = 6000


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from macaw_gb300 import problems
    from oracle.oracle import Oracle
    p = problems.lattice_problem(nx=3, ny=3, nz=3, height=6.0, n_pts=1500)
    o = Oracle(p)
    per = N // world
    tally, traces, st, _ = o.run(per, first=rank * per, seed=3, threads=1)
    t = torch.from_numpy(tally)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    hashes = torch.from_numpy(traces["hash"].view(np.int64).copy())
    gathered = [torch.zeros_like(hashes) for _ in range(world)]
    dist.all_gather(gathered, hashes)
    nseg = torch.tensor([st["n_seg"]], dtype=torch.int64)
    dist.all_reduce(nseg, op=dist.ReduceOp.SUM)
    if rank == 0:
        np.save(os.path.join(out_dir, "tally.npy"), t.numpy())
        np.save(os.path.join(out_dir, "hash.npy"), torch.cat(gathered).numpy())
        np.save(os.path.join(out_dir, "nseg.npy"), nseg.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharding_equals_single_rank(tmp_path):
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    from macaw_gb300 import problems
    from oracle.oracle import Oracle
    p = problems.lattice_problem(nx=3, ny=3, nz=3, height=6.0, n_pts=1500)
    tally, traces, st, _ = Oracle(p).run(N, seed=3, threads=1)
    got_t = np.load(tmp_path / "tally.npy")
    got_h = np.load(tmp_path / "hash.npy")
    assert np.array_equal(got_h, traces["hash"].view(np.int64))
    nz = tally != 0
    assert np.all(np.abs(got_t[nz] - tally[nz]) <= 1e-12 * tally[nz])
    assert int(np.load(tmp_path / "nseg.npy")[0]) == st["n_seg"]
