"""Multi-GPU execution of run(): FFT blocks shard across ranks, results are summed once.

The reference distributes K-points over Ray workers and sums their results on the host
(run_grid.py:59-66,79-109).  Here one process drives one GPU: each rank integrates a contiguous
shard of the division-grid blocks with the ordinary single-GPU run() (no collective inside the
data path), and the per-calculator results -- each already carrying the 1/prod(NKdiv) block
weight -- are summed across ranks with one all-reduce of their data arrays.  Works with any
torch.distributed backend (NCCL on GPUs, gloo on CPU for the host-logic tests).
"""
import numpy as np
import torch

from .result import EnergyResult, ResultDict


def shard_blocks(nblocks, rank, world):
    """Contiguous shard of block indices [0, nblocks) for `rank` of `world` (sizes differ by at
    most one; every block belongs to exactly one rank)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    base, extra = divmod(int(nblocks), int(world))
    start = rank * base + min(rank, extra)
    return np.arange(start, start + base + (1 if rank < extra else 0))


def allreduce_results(results, group=None):
    """Sum a ResultDict of EnergyResults over the ranks of `group` (all ranks return the sum).
    Every rank must hold the same keys and array shapes (the calculators are identical)."""
    out = ResultDict()
    for key in sorted(results):
        r = results[key]
        data = np.asarray(r.data)
        if np.iscomplexobj(data):
            t = torch.from_numpy(np.ascontiguousarray(np.stack([data.real, data.imag])).astype(np.float64))
        else:
            t = torch.from_numpy(np.ascontiguousarray(data, dtype=np.float64))
        if torch.distributed.get_backend(group) == 'nccl':
            t = t.cuda()
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM, group=group)
        t = t.cpu().numpy()
        summed = t[0] + 1j * t[1] if np.iscomplexobj(data) else t
        out[key] = EnergyResult(r.Energies[0] if len(r.Energies) == 1 else r.Energies, summed,
                                comment=getattr(r, 'comment', ''))
    return out


def run_sharded(system, grid, calculators, run_fn=None, group=None, **kwargs):
    """run() over this rank's shard of the grid's blocks, then the cross-rank sum.  `run_fn`
    defaults to wbgpu.run (GPU); it receives (system, grid, calculators, blocks=..., **kwargs)."""
    if run_fn is None:
        from .run import run as run_fn
    world = torch.distributed.get_world_size(group)
    rank = torch.distributed.get_rank(group)
    mine = shard_blocks(grid.nblocks, rank, world)
    res = run_fn(system, grid, calculators, blocks=mine, **kwargs)
    return allreduce_results(res, group)
