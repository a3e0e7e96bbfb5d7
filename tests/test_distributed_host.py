"""Multi-rank host logic on CPU (gloo, world size 2): blocks shard across ranks with no
collective in the data path, and the per-calculator results are summed once.  Each rank runs
the oracle on its shard; the sum must equal one single-process run over all blocks."""
import os
import random

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from oracle import wb_oracle as O
from wbgpu import models
from wbgpu.distributed import shard_blocks, allreduce_results, run_sharded

NKDIV, NKFFT = (3, 2, 2), (2, 3, 2)
EF = np.linspace(-1.5, 1.5, 13)


class _Grid:
    nblocks = int(np.prod(NKDIV))


def _system():
    d = models.config_system(1, small=True)
    return O.RSystem(d['real_lattice'], d['iRvec'], d['wannier_centers_cart'], d['XX_R'])


def _oracle_run(system, grid, calculators, blocks):
    return O.run(system, NKDIV, NKFFT, calculators, blocks=blocks)


def _worker(rank, world, port, path):
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    torch.distributed.init_process_group('gloo', rank=rank, world_size=world)
    try:
        calcs = {'ahc': O.AHC(Efermi=EF), 'opt': O.OpticalConductivity(Efermi=EF[::4], omega=np.linspace(0.1, 1, 5))}
        res = run_sharded(_system(), _Grid(), calcs, run_fn=_oracle_run)
        np.savez(f"{path}_{rank}.npz", ahc=res['ahc'].data, opt=res['opt'].data)
    finally:
        torch.distributed.destroy_process_group()


def test_shard_blocks_partition():
    for nb in (1, 5, 27, 512):
        for world in (1, 2, 3, 8):
            parts = [shard_blocks(nb, r, world) for r in range(world)]
            assert np.array_equal(np.concatenate(parts), np.arange(nb))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_blocks(4, 2, 2)


def test_two_ranks_gloo_sum_equals_single_run(tmp_path):
    port = random.randint(20000, 40000)
    path = str(tmp_path / "res")
    mp.spawn(_worker, args=(2, port, path), nprocs=2, join=True)
    full = O.run(_system(), NKDIV, NKFFT, {'ahc': O.AHC(Efermi=EF),
                                           'opt': O.OpticalConductivity(Efermi=EF[::4], omega=np.linspace(0.1, 1, 5))})
    for rank in (0, 1):  # every rank holds the sum
        got = np.load(f"{path}_{rank}.npz")
        for key in ('ahc', 'opt'):
            ref = full[key].data
            assert np.abs(got[key] - ref).max() <= 1e-12 * np.abs(ref).max(), (rank, key)


def test_allreduce_single_rank_identity(tmp_path):
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(random.randint(40001, 50000))
    torch.distributed.init_process_group('gloo', rank=0, world_size=1)
    try:
        r = O.run(_system(), NKDIV, NKFFT, {'ahc': O.AHC(Efermi=EF)})
        s = allreduce_results(r)
        assert np.array_equal(s['ahc'].data, r['ahc'].data)
    finally:
        torch.distributed.destroy_process_group()
