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


def more_batches_of_size(nblocks, nb, i0):
    """Whether the batch of `nblocks` blocks split into batches of `nb` that starts at block `i0`
    is followed by another batch of the same size (the full batches all are, except the last)."""
    n_this = min(nb, nblocks - i0)
    return nblocks - (i0 + n_this) >= n_this


def block_results(dev, system, shifts, NKFFT, calculators, precision, cells=None):
    """One result per block -- what the reference's calculators return for one Data_K (normalised
    by the block's k-points, K-point factor 1): [{key: EnergyResult}] for the blocks at `shifts`.
    Each block gets fresh copies of the calculators; batches of blocks share stages 1-3.
    `cells`: each block's dense-grid cell (dK_block / NKFFT), for tetrahedron calculators."""
    quantities = set()
    for c in calculators.values():
        quantities |= c.quantities(system)
    tetra = any(getattr(c, 'tetra', False) for c in calculators.values())
    if tetra and cells is None:
        raise ValueError("tetra=True needs the cell of every block")
    nk = int(np.prod(NKFFT))
    nb = choose_batch(dev.nw, nk, len(shifts), quantities, precision)
    out = []
    for i0 in range(0, len(shifts), nb):
        corners = None
        if tetra:  # computed before band_data: both use the system's default workspace
            corners = engine.BlockCorners(dev, shifts[i0:i0 + nb], cells[i0:i0 + nb], NKFFT, precision)
        bd = engine.band_data(dev, shifts[i0:i0 + nb], NKFFT, quantities, precision)
        if corners is not None:
            corners.attach(bd, np.arange(bd.nblocks))
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
        if corners is not None:
            corners.check()
    return out


class Refinement:
    """The reference's adaptive refinement without symmetry (run_grid.py:290-403; Kpoint.divide at
    grid/Kpoint.py:145-175) on a K-point list: after each round of evaluations all K-points are
    ranked by max(result) x factor per entry of ResultDict.max, the adpt_fac largest of each entry
    are divided into prod(adpt_mesh) sub-blocks (periodic directions only) with factor /
    prod(adpt_mesh), and the parent's factor is set to 0."""

    def __init__(self, system, grid, calculators, adpt_num_iter, adpt_mesh=2, adpt_fac=1):
        self.div, self.fft = np.array(grid.div, dtype=int), np.array(grid.FFT, dtype=int)
        if adpt_num_iter < 0:
            adpt_num_iter = -adpt_num_iter * np.prod(self.div) / np.prod(adpt_mesh) / adpt_fac / 3
        self.num_iter = int(round(adpt_num_iter))
        self.mesh = np.array(adpt_mesh, dtype=int) * np.ones(3, dtype=int)
        if self.mesh.max() <= 1:
            self.num_iter = 0
        self.fac_top = int(adpt_fac)
        self.periodic = np.array(getattr(system, 'periodic', (True, True, True)), dtype=bool)
        self.templates = {k: copy.deepcopy(c) for k, c in calculators.items()}
        idx = np.stack(np.meshgrid(*[np.arange(n) for n in self.div], indexing='ij'), axis=-1).reshape(-1, 3)
        self.K = list(idx / self.div[None, :])
        self.dK = [1.0 / self.div for _ in self.K]
        self.fac = [1.0 / np.prod(self.div) for _ in self.K]
        self.results = []
        self.it = 0

    def new_shifts(self):
        """Block shifts dK = K / NKFFT of the K-points not evaluated yet."""
        return np.array(self.K[len(self.results):]) / self.fft[None, :]

    def new_cells(self):
        """Dense-grid cells dK / NKFFT of those K-points (the tetrahedra's parallelepipeds)."""
        return np.array(self.dK[len(self.results):]) / self.fft[None, :]

    def add(self, results):
        self.results += list(results)

    def refine(self):
        """Divide the selected K-points; False when the last iteration has been evaluated."""
        if self.it >= self.num_iter:
            return False
        self.it += 1
        Kmax = np.array([np.concatenate([r[key].max for key in self.templates]) * f
                         for r, f in zip(self.results, self.fac)]).T
        select = set().union(*(np.argsort(km)[-self.fac_top:] for km in Kmax))
        for iK in select:
            nd = self.mesh.copy()
            nd[~self.periodic] = 1
            dka = self.dK[iK] / nd
            shift = (-self.dK[iK] + dka) / 2.0
            for x in range(nd[0]):
                for y in range(nd[1]):
                    for z in range(nd[2]):
                        self.K.append(self.K[iK] + shift + dka * np.array([x, y, z]))
                        self.dK.append(dka)
                        self.fac.append(self.fac[iK] / np.prod(nd))
            self.fac[iK] = 0.0
        return True

    def total(self):
        out = {}
        for r, f in zip(self.results, self.fac):
            for key in self.templates:
                out[key] = r[key] * f if key not in out else out[key] + r[key] * f
        return ResultDict(out)


def run_adaptive(system, grid, calculators, precision, dev, adpt_num_iter, adpt_mesh=2, adpt_fac=1):
    """run() with adaptive refinement (Refinement): returns (ResultDict, K, dK, factor)."""
    ref = Refinement(system, grid, calculators, adpt_num_iter, adpt_mesh, adpt_fac)
    while True:
        ref.add(block_results(dev, system, ref.new_shifts(), ref.fft, ref.templates, precision, ref.new_cells()))
        if not ref.refine():
            break
    return ref.total(), np.array(ref.K), np.array(ref.dK), np.array(ref.fac)


def run(system, grid, calculators, precision='fp64', blocks_per_batch=None, device='cuda', dev_system=None,
        blocks=None, adpt_num_iter=0, adpt_mesh=2, adpt_fac=1, cuda_graph=False, autotune=False, **_ignored):
    """Integrate ``calculators`` over ``grid``.  precision: 'fp64' (plain) or 'mixed'
    (double-float H(k) and eigh, FP64 scan, FP32 fields and rotations).  ``blocks`` restricts the
    run to a subset of the division-grid K-points (indices into Grid.block_shifts());
    the result then carries the same 1/prod(NKdiv) weight per block.  ``adpt_num_iter`` > 0:
    adaptive refinement with the reference's policy (``adpt_mesh``, ``adpt_fac``).
    ``cuda_graph``: stages 1-3 of every batch after the first two of a shape are replayed from
    a CUDA graph (engine.band_data_graphed; bit-identical results, fewer host calls per batch).
    The eigensolver's convergence flags are read once, after the last batch, so the host queues
    batch after batch without waiting for the device.
    ``autotune``: launch shapes of the eigensolver and the rotation for this num_wann and
    precision from the autotuner (wbgpu.autotune.ensure: cached per device, measured once)."""
    engine.require_cuda()
    dev = dev_system or engine.DeviceSystem(system, device)
    if autotune:
        from . import autotune as _tune
        _tune.ensure(dev.nw, precision, device=dev.device)
    if adpt_num_iter:
        if blocks is not None:
            raise ValueError("adaptive refinement runs over the whole grid (blocks must be None)")
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
    precs = engine.phase_precs(precision)
    phases = {p: dev.grid_phases(shifts, grid.FFT, p) for p in precs}
    flags = []
    for i0 in range(0, len(shifts), nb):
        if cuda_graph:  # a graph is captured only when a later batch of this size will replay it
            bd = engine.band_data_graphed(dev, shifts[i0:i0 + nb], grid.FFT, quantities, precision, phases=phases,
                                          block_start=i0, more=more_batches_of_size(len(shifts), nb, i0))
        else:
            bd = engine.band_data(dev, shifts[i0:i0 + nb], grid.FFT, quantities, precision, phases=phases,
                                  block_start=i0)
        if tetra is not None:
            tetra.attach(bd, block_ids[i0:i0 + nb])
        for c in calculators.values():
            c.accumulate(bd, system)
        flags.append(bd._flag.clone())  # the batch's QL flag (its buffer is reused by the next batch)
        del bd
    engine.check_flags(flags)
    if tetra is not None:
        tetra.check()
    factor = 1.0 / grid.nblocks
    return ResultDict({k: c.result(system.cell_volume, nk, factor) for k, c in calculators.items()})
