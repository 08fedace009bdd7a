"""Multi-GPU layout of the basis computation: one process per GPU, each
owning its own coarse cells, no collective on the data path.

The reference distributes coarse cells over MPI ranks with p4est
(include/base/diffusion_problem_ms.tpp:50-58) and its basis phase never
communicates (each rank computes the basis of its locally owned cells,
:81-87).  The same holds here: a rank's cells, coefficient and outputs stay
on its GPU; the only cross-rank operation is the reduction of the timing
(the slowest rank defines the job's time) and the sum of work counts.
"""
import numpy as np


def weak_shard_corners(corners, rank):
    """Weak scaling: rank r owns its own copy of the coarse mesh block moved by
    r along x (the unit square [r, r+1] x [0, 1]), so per-rank work is fixed
    and the coefficient differs between ranks."""
    c = np.ascontiguousarray(corners, dtype=np.float64)
    shift = np.zeros(c.shape[-1])
    shift[0] = float(rank)
    return np.ascontiguousarray(c + shift)


def block_partition(n_cells, world, rank):
    """Strong scaling: contiguous blocks of cells, sizes differing by at most
    one ([start, stop) of `rank`), as p4est's space-filling-curve partition
    gives contiguous locally owned ranges."""
    base, extra = divmod(int(n_cells), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def assemble_blocks(blocks, n_cells):
    """Per-cell arrays of a strongly sharded batch from every rank's block:
    blocks = [(start, stop, [array, ...]), ...] (arrays with leading dimension
    stop - start).  Every cell must be owned by exactly one block."""
    owner = np.zeros(int(n_cells), dtype=np.int64)
    out = None
    for start, stop, arrays in blocks:
        owner[start:stop] += 1
        if out is None:
            out = [np.zeros((int(n_cells),) + np.asarray(a).shape[1:], dtype=np.asarray(a).dtype) for a in arrays]
        for o, a in zip(out, arrays):
            o[start:stop] = a
    if not np.all(owner == 1):
        raise ValueError("cells owned by no rank or by several: "
                         f"{np.flatnonzero(owner != 1)[:8].tolist()}")
    return out


def gather_blocks(arrays, start, stop, n_cells, dist=None):
    """Outputs of a strongly sharded batch on every rank (the host-side
    all-gather of each rank's [start, stop) block; the basis computation
    itself exchanges nothing).  Identity at one rank."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return assemble_blocks([(start, stop, arrays)], n_cells)
    blocks = [None] * dist.get_world_size()
    dist.all_gather_object(blocks, (int(start), int(stop), [np.asarray(a) for a in arrays]))
    return assemble_blocks(blocks, n_cells)


def max_over_ranks(value, dist=None, device="cpu"):
    """Job time = the slowest rank's time (a MAX all-reduce; identity at 1 rank)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, dist=None, device="cpu"):
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def job_throughput(units_all_ranks, seconds_max):
    """Whole-job rate: the units every rank processed over the slowest rank's time."""
    return float(units_all_ranks) / float(seconds_max)
