"""run() mirror (run_grid.py:118-403): integrate calculators over a Grid on the GPU.

Blocks (K-points of the division grid) are processed in batches; each batch runs
stages 1-3 once (engine.band_data) and every calculator accumulates its device
histogram from the same band data.  Results are summed over blocks times the K-point
factor 1/prod(NKdiv) (run_grid.py:59-66).  No symmetry reduction, refinement or
restart files (those live outside the GPU hot path).  Calculators with tetra=True get
the corner energies of the tetrahedron method (engine.TetraCorners), computed once per run.
"""
import numpy as np
import torch

from . import engine
from .result import ResultDict


def choose_batch(nw, nk, nblocks, quantities, precision, max_kpoints=1 << 17, budget_bytes=24 << 30):
    cs = 16 if precision == 'fp64' else 8
    nf = 1 + sum(engine.QUANTITIES[q]['ncomp'] for q in quantities)
    per_k = nw * nw * (2 * nf * cs + 16 * 3) + 64 * nw
    nb = max(1, min(nblocks, max_kpoints // nk, budget_bytes // max(per_k * nk * 3, 1)))
    return int(nb)


def run(system, grid, calculators, precision='fp64', blocks_per_batch=None, device='cuda', dev_system=None,
        blocks=None, **_ignored):
    """Integrate ``calculators`` over ``grid``.  precision: 'fp64' (plain) or 'mixed'
    (double-float H(k) and eigh, FP64 scan, FP32 fields and rotations).  ``blocks`` restricts the
    run to a subset of the division-grid K-points (indices into Grid.block_shifts());
    the result then carries the same 1/prod(NKdiv) weight per block."""
    engine.require_cuda()
    dev = dev_system or engine.DeviceSystem(system, device)
    quantities = set()
    for c in calculators.values():
        quantities |= c.quantities(system)
    for c in calculators.values():
        c.reset(dev.device)
    shifts = grid.block_shifts()
    block_ids = np.arange(len(shifts)) if blocks is None else np.asarray(blocks, dtype=int)
    shifts = shifts[block_ids]
    nk = grid.nk_per_block
    nb = blocks_per_batch or choose_batch(dev.nw, nk, len(shifts), quantities, precision)
    # tetrahedron method: corner energies of every block the run touches, once, kept resident
    tetra = None
    if any(getattr(c, 'tetra', False) for c in calculators.values()):
        tetra = engine.TetraCorners(dev, grid, block_ids, precision)
    precs = [engine.PREC_FP64] if precision == 'fp64' else [engine.PREC_DF64, engine.PREC_FP32S]
    phases = {p: dev.grid_phases(shifts, grid.FFT, p) for p in precs}
    for i0 in range(0, len(shifts), nb):
        bd = engine.band_data(dev, shifts[i0:i0 + nb], grid.FFT, quantities, precision, phases=phases,
                              block_start=i0)
        if tetra is not None:
            tetra.attach(bd, block_ids[i0:i0 + nb])
        for c in calculators.values():
            c.accumulate(bd, system)
        engine.check_flag(bd)
        del bd
    if tetra is not None:
        tetra.check()
    factor = 1.0 / grid.nblocks
    return ResultDict({k: c.result(system.cell_volume, nk, factor) for k, c in calculators.items()})
