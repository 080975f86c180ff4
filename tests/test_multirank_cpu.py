"""Multi-rank sharding of histories (world_size 2, gloo, CPU).

Across GPUs the path shards by history index: rank r tracks a disjoint
range of particle ids, and the only exchange is one FP64 sum-reduce of the
element tallies at the end.  Because every history's random numbers are
keyed by its global id, the sharded result must equal a single-rank run:
per-history traces identical, tallies equal up to summation order.  The
ranks here split the histories with the library's history_range and sum
the tallies with its reduce_tally (macaw_gb300/shard.py) over gloo; each
rank tracks its range with the oracle on the CPU.  The library's own
tracker on both halves of a range is tests/test_gpu_shard.py.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

N = 6001  # uneven: rank 0 tracks one history more


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from macaw_gb300 import problems
    from macaw_gb300.shard import history_range, reduce_tally
    from oracle.oracle import Oracle
    p = problems.lattice_problem(nx=3, ny=3, nz=3, height=6.0, n_pts=1500)
    o = Oracle(p)
    first, per = history_range(N, rank, world)
    tally, traces, st, _ = o.run(per, first=first, seed=3, threads=1)
    t = torch.from_numpy(reduce_tally(tally))
    hashes = torch.zeros(N // world + 1, dtype=torch.int64)
    hashes[:per] = torch.from_numpy(traces["hash"].view(np.int64).copy())
    gathered = [torch.zeros_like(hashes) for _ in range(world)]
    dist.all_gather(gathered, hashes)
    gathered = [g[:history_range(N, r, world)[1]] for r, g in enumerate(gathered)]
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


def test_history_range_partitions():
    from macaw_gb300.shard import history_range
    for n in (0, 1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            parts = [history_range(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and sum(c for _, c in parts) == n
            for (f0, c0), (f1, _) in zip(parts, parts[1:]):
                assert f0 + c0 == f1
            assert max(c for _, c in parts) - min(c for _, c in parts) <= 1


def test_reduce_tally_without_a_group_is_the_identity():
    from macaw_gb300.shard import reduce_tally
    a = np.arange(5, dtype=np.float64)
    assert reduce_tally(a) is a
