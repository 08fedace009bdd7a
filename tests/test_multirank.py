"""The N > 1 host path on CPU: two gloo ranks (127.0.0.1) run the same
sharding and timing-reduction code bench.py runs under torchrun with NCCL.

Checked: weak-scaling shards are disjoint copies of the coarse mesh (no cell
owned twice, no data exchanged), strong-scaling blocks cover every cell
exactly once, the job time is the slowest rank's, and the job rate counts
every rank's units over that time.  And the sharded computation itself: each
rank solves the basis problems of its own block of coarse cells (the CPU
oracle stands in for the GPU, which this test does not need), and the
gathered blocks equal the one-rank batch bit for bit, every cell owned once."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    import __graft_entry__ as graft

    pkg = graft.load_package()
    S, W = pkg.sharding, pkg.workloads
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        corners = S.weak_shard_corners(W.unit_cube_corners(2, 8), rank)
        lo, hi = corners.reshape(-1, 2).min(axis=0), corners.reshape(-1, 2).max(axis=0)
        start, stop = S.block_partition(1000, world, rank)
        t_ms = [3.0, 5.0][rank]
        t_max = S.max_over_ranks(t_ms, dist)
        units = S.sum_over_ranks(4 * corners.shape[0], dist)
        rate = S.job_throughput(units, t_max * 1e-3)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), lo=lo, hi=hi, start=start, stop=stop,
                 t_max=t_max, units=units, rate=rate, corners=corners)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    r = [dict(np.load(tmp_path / f"rank{k}.npz")) for k in range(world)]
    # weak scaling: rank k owns [k, k+1] x [0, 1]; the blocks touch but do not overlap
    for k in range(world):
        assert np.allclose(r[k]["lo"], [k, 0.0]) and np.allclose(r[k]["hi"], [k + 1, 1.0])
    cells0 = {tuple(np.round(c.mean(axis=0), 12)) for c in r[0]["corners"]}
    cells1 = {tuple(np.round(c.mean(axis=0), 12)) for c in r[1]["corners"]}
    assert not cells0 & cells1
    # strong scaling: contiguous blocks cover [0, 1000) once
    assert int(r[0]["start"]) == 0 and int(r[0]["stop"]) == int(r[1]["start"]) and int(r[1]["stop"]) == 1000
    # the job time is the slowest rank's on every rank; the rate counts all units
    for k in range(world):
        assert float(r[k]["t_max"]) == 5.0
        assert float(r[k]["units"]) == 2 * 4 * 64
        assert float(r[k]["rate"]) == pytest.approx(2 * 4 * 64 / 5e-3)


def _solve_worker(rank, world, port, out_dir):
    import torch.distributed as dist

    import __graft_entry__ as graft

    pkg, oracle = graft.load_package(), graft.load_oracle()
    S, W = pkg.sharding, pkg.workloads
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        prob = W.sinsin_square()  # 8 x 8 coarse cells, N = 16: the CPU-runnable configuration
        n = prob["corners"].shape[0]
        start, stop = S.block_partition(n, world, rank)
        res = oracle.run(W.subset(prob, np.arange(start, stop)), tol=1e-12)
        M, F = S.gather_blocks([res["M"], res["F"]], start, stop, n, dist)
        if rank == 0:
            np.savez(os.path.join(out_dir, "gathered.npz"), M=M, F=F)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_basis_equals_one_rank(pkg, oracle, tmp_path, world):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    mp.spawn(_solve_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    got = dict(np.load(tmp_path / "gathered.npz"))
    one = oracle.run(pkg.workloads.sinsin_square(), tol=1e-12)
    assert np.array_equal(got["M"], one["M"])
    assert np.array_equal(got["F"], one["F"])


def test_gather_blocks_rejects_overlap(pkg):
    """A cell claimed by two ranks (or by none) is an error, not a silent overwrite."""
    S = pkg.sharding
    with pytest.raises(ValueError):
        S.assemble_blocks([(0, 3, [np.zeros((3, 2))]), (2, 4, [np.zeros((2, 2))])], 4)
    with pytest.raises(ValueError):
        S.assemble_blocks([(0, 1, [np.zeros((1, 2))]), (2, 4, [np.zeros((2, 2))])], 4)


@pytest.mark.parametrize("n,world", [(10, 3), (7, 7), (5, 8), (4096, 4)])
def test_block_partition_covers_every_cell_once(pkg, n, world):
    S = pkg.sharding
    blocks = [S.block_partition(n, world, r) for r in range(world)]
    assert blocks[0][0] == 0 and blocks[-1][1] == n
    for (a, b), (c, d) in zip(blocks, blocks[1:]):
        assert b == c
    sizes = [b - a for a, b in blocks]
    assert max(sizes) - min(sizes) <= 1
