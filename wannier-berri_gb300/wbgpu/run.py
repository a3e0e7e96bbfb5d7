"""run() mirror (run_grid.py:118-403): integrate calculators over a Grid on the GPU.

Blocks (K-points of the division grid) are processed in batches; each batch runs
stages 1-3 once (engine.band_data) and every calculator accumulates its device
histogram from the same band data.  Results are summed over blocks times the K-point
factor 1/prod(NKdiv) (run_grid.py:59-66).  Adaptive refinement (adpt_num_iter) follows the
reference's policy without symmetry (run_adaptive); no symmetry reduction or restart files.
Calculators with tetra=True get the corner energies of the tetrahedron method
(engine.TetraCorners), computed once per run.
"""
import copy

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


def block_results(dev, system, shifts, NKFFT, calculators, precision, dk_cell=None):
    """One result per block -- what the reference's calculators return for one Data_K (normalised
    by the block's k-points, K-point factor 1): [{key: EnergyResult}] for the blocks at `shifts`.
    Each block gets fresh copies of the calculators; batches of blocks share stages 1-3."""
    quantities = set()
    for c in calculators.values():
        quantities |= c.quantities(system)
    nk = int(np.prod(NKFFT))
    nb = choose_batch(dev.nw, nk, len(shifts), quantities, precision)
    out = []
    for i0 in range(0, len(shifts), nb):
        bd = engine.band_data(dev, shifts[i0:i0 + nb], NKFFT, quantities, precision)
        for b in range(bd.nblocks):
            sub = bd.block(b)
            res = {}
            for key, c in calculators.items():
                cb = copy.deepcopy(c)
                cb.reset(dev.device)
                cb.accumulate(sub, system)
                res[key] = cb.result(system.cell_volume, nk, 1.0)
            out.append(res)
        engine.check_flag(bd)
    return out


def run_adaptive(system, grid, calculators, precision, dev, adpt_num_iter, adpt_mesh=2, adpt_fac=1):
    """run() with adaptive refinement, without symmetry (run_grid.py:290-403; Kpoint.divide at
    grid/Kpoint.py:145-175): each iteration evaluates the new K-points (blocks), ranks all
    K-points by max(result) x factor per entry of ResultDict.max, divides the adpt_fac largest
    of each entry into prod(adpt_mesh) sub-blocks with factor / prod(adpt_mesh) (along periodic
    directions only) and sets the parent's factor to 0.  Returns (ResultDict, K, dK, factor)."""
    div, fft = np.array(grid.div, dtype=int), np.array(grid.FFT, dtype=int)
    if adpt_num_iter < 0:
        adpt_num_iter = -adpt_num_iter * np.prod(div) / np.prod(adpt_mesh) / adpt_fac / 3
    adpt_num_iter = int(round(adpt_num_iter))
    mesh = np.array(adpt_mesh, dtype=int) * np.ones(3, dtype=int)
    if mesh.max() <= 1:
        adpt_num_iter = 0
    templates = {k: copy.deepcopy(c) for k, c in calculators.items()}
    idx = np.stack(np.meshgrid(*[np.arange(n) for n in div], indexing='ij'), axis=-1).reshape(-1, 3)
    K = list(idx / div[None, :])
    dK = [1.0 / div for _ in K]
    fac = [1.0 / np.prod(div) for _ in K]
    res = []
    periodic = np.array(getattr(system, 'periodic', (True, True, True)), dtype=bool)
    for it in range(adpt_num_iter + 1):
        new = np.array(K[len(res):])
        res += block_results(dev, system, new / fft[None, :], fft, templates, precision)
        if it >= adpt_num_iter:
            break
        Kmax = np.array([np.concatenate([r[key].max for key in templates]) * f for r, f in zip(res, fac)]).T
        select = set().union(*(np.argsort(km)[-adpt_fac:] for km in Kmax))
        for iK in select:
            nd = mesh.copy()
            nd[~periodic] = 1
            dka = dK[iK] / nd
            shift = (-dK[iK] + dka) / 2.0
            for x in range(nd[0]):
                for y in range(nd[1]):
                    for z in range(nd[2]):
                        K.append(K[iK] + shift + dka * np.array([x, y, z]))
                        dK.append(dka)
                        fac.append(fac[iK] / np.prod(nd))
            fac[iK] = 0.0
    total = {}
    for r, f in zip(res, fac):
        for key in templates:
            total[key] = r[key] * f if key not in total else total[key] + r[key] * f
    return ResultDict(total), np.array(K), np.array(dK), np.array(fac)


def run(system, grid, calculators, precision='fp64', blocks_per_batch=None, device='cuda', dev_system=None,
        blocks=None, adpt_num_iter=0, adpt_mesh=2, adpt_fac=1, **_ignored):
    """Integrate ``calculators`` over ``grid``.  precision: 'fp64' (plain) or 'mixed'
    (double-float H(k) and eigh, FP64 scan, FP32 fields and rotations).  ``blocks`` restricts the
    run to a subset of the division-grid K-points (indices into Grid.block_shifts());
    the result then carries the same 1/prod(NKdiv) weight per block.  ``adpt_num_iter`` > 0:
    adaptive refinement with the reference's policy (``adpt_mesh``, ``adpt_fac``)."""
    engine.require_cuda()
    dev = dev_system or engine.DeviceSystem(system, device)
    if adpt_num_iter:
        if blocks is not None:
            raise ValueError("adaptive refinement runs over the whole grid (blocks must be None)")
        if any(getattr(c, 'tetra', False) for c in calculators.values()):
            raise NotImplementedError("tetra=True with adaptive refinement is not supported by the GPU backend")
        return run_adaptive(system, grid, calculators, precision, dev, adpt_num_iter, adpt_mesh, adpt_fac)[0]
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
