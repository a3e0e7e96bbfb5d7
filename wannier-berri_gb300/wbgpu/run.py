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


# ---------------------------------------------------------------------------------------
# Refinement around the largest Berry curvatures: the top fraction of the k-points by
# max_n |Omega_n(k)| get a mesh^3 sub-grid of their cell, round after round.
# ---------------------------------------------------------------------------------------
def subgrid_shifts(points, cell, mesh):
    """Block shifts of mesh^3 sub-grids centred on `points` (n, 3) whose cells have edges `cell`
    (3,): the sub-grid of k has the points k + (j - (mesh - 1) / 2) cell / mesh, j = 0..mesh-1 per
    axis (the midpoints of the mesh^3 sub-cells), i.e. shift k - (mesh - 1) / 2 step and per-axis
    step = cell / mesh.  Returns (shifts, step)."""
    step = np.asarray(cell, dtype=float) / mesh
    return np.asarray(points, dtype=float) - 0.5 * (mesh - 1) * step[None, :], step


def block_points(shifts, NKFFT, step, index):
    """Coordinates of the k-points `index` (flat: block-major, C order of the block's NKFFT points)
    of blocks with `shifts` and per-axis `step`."""
    nk = int(np.prod(NKFFT))
    index = np.asarray(index, dtype=np.int64)
    b, j = index // nk, index % nk
    ijk = np.stack(np.unravel_index(j, tuple(int(n) for n in NKFFT)), axis=-1)
    return np.asarray(shifts, dtype=float)[b] + ijk * np.asarray(step, dtype=float)[None, :]


def _omega_scores(bd, degen_thresh):
    """max over bands of |Omega_n(k)| (group-averaged Berry curvature, the tabulation kernel of
    wbg_berry_tabulate) for every k-point of a batch."""
    import ctypes
    from . import _lib
    from .engine import _ptr, _stream
    tab = torch.empty((bd.nk_total, bd.nw, 7), dtype=torch.float64, device=bd.E.device)
    ext = 1 if 'A' in bd.index else 0
    st = _lib.load().wbg_berry_tabulate(_ptr(bd.E), _ptr(bd.Xbar), bd.Xbar.shape[1], bd.index['V'],
                                        bd.index.get('A', 0), bd.index.get('Od', 0), bd.nw, bd.nk_total,
                                        ctypes.c_double(degen_thresh), 1, ext, _ptr(tab), int(bd.fp64_fields),
                                        _stream())
    _lib.check(st, "wbg_berry_tabulate")
    return tab[:, :, 4:7].norm(dim=2).amax(dim=1)


def _evaluate_blocks(dev, system, shifts, NKFFT, step, calculators, quantities, precision, scores,
                     degen_thresh=1e-4, cached_phases=True):
    """Stages 1-3 and every calculator over blocks of NKFFT points (spacing `step`, None: 1/NKFFT)
    at `shifts`; with `scores` the per-k Berry-curvature scores of the blocks in order (device)."""
    nk = int(np.prod(NKFFT))
    nb = choose_batch(dev.nw, nk, len(shifts), quantities, precision)
    keep, phases = [], {}
    for p in engine.phase_precs(precision):
        if cached_phases:
            phases[p] = dev.grid_phases(shifts, NKFFT, p, step=step)
        else:
            phases[p], host = dev.grid_phases(shifts, NKFFT, p, step=step, cache=False)
            keep.append(host)
    out, flags = [], []
    for i0 in range(0, len(shifts), nb):
        bd = engine.band_data(dev, shifts[i0:i0 + nb], NKFFT, quantities, precision, phases=phases, block_start=i0)
        for c in calculators.values():
            c.accumulate(bd, system)
        if scores:
            out.append(_omega_scores(bd, degen_thresh))
        flags.append(bd._flag.clone())
        del bd
    engine.check_flags(flags)
    return torch.cat(out) if scores else None


class _Job:
    """Blocks of one kind within a refinement round: NKFFT points spaced by `step` (None: the
    FFT grid) at `shifts`, accumulated by `calcs`; their results enter with weight `factor` per
    block of `nk` points and `sign`."""

    def __init__(self, shifts, fft, step, calcs, scores, nk, factor, sign):
        self.shifts, self.fft, self.step, self.calcs = np.asarray(shifts, dtype=float), tuple(fft), step, calcs
        self.scores, self.nk, self.factor, self.sign = scores, nk, factor, sign


class OmegaRefinement:
    """Refinement around the largest Berry curvatures, round by round.  Round 0 is the grid; after
    each round, top x (k-points of the grid) of its scored k-points (the grid's, then the previous
    round's sub-grid points) with the largest max_n |Omega_n(k)| are each replaced by a mesh^3
    sub-grid of their cell (subgrid_shifts): every round refines as many points as the first.  The result is the grid's sum with each refined point's value
    replaced by the mean of its sub-grid: per refined point k of weight w (1/N for a point of the
    grid of N k-points, w / mesh^3 one round further), w (mean over the sub-grid - value at k).
    Refining every point (top = 1) gives the grid with mesh times more points per axis, shifted by
    half a sub-cell.  jobs() lists the current round's blocks; end_round(scores) takes the
    round's per-k scores (of the scored job, in block order) and plans the next round."""

    def __init__(self, system, grid, calculators, device, rounds=1, top=0.01, mesh=8):
        if any(getattr(c, 'tetra', False) for c in calculators.values()):
            raise NotImplementedError("refinement around the largest Berry curvatures does not take tetra=True")
        if not top > 0.0 or mesh < 1 or rounds < 0:
            raise ValueError("top must be > 0 (refined points per round / points of the grid), mesh >= 1, "
                             "rounds >= 0")
        self.system, self.templates, self.device = system, calculators, device
        self.rounds, self.top, self.mesh = int(rounds), float(top), int(mesh)
        self.quantities = set()
        for c in calculators.values():
            self.quantities |= c.quantities(system)
        ext = system.has_R_mat('AA') and not system.force_internal_terms_only
        self.quantities |= {'V', 'A', 'Od'} if ext else {'V'}
        fft = np.array(grid.FFT, dtype=int)
        npts = fft * np.array(grid.div, dtype=int)
        self.cell, self.weight = 1.0 / npts, 1.0 / float(np.prod(npts))
        self.round = 0
        self.total = {}
        self._jobs = [_Job(grid.block_shifts(), fft, None, self._fresh(), self.rounds > 0, int(np.prod(fft)),
                           1.0 / grid.nblocks, 1.0)]
        self.kpoints = self.n_grid = grid.nblocks * int(np.prod(fft))

    def _fresh(self):
        cs = {k: copy.deepcopy(c) for k, c in self.templates.items()}
        for c in cs.values():
            c.reset(self.device)
        return cs

    def jobs(self):
        return self._jobs

    def end_round(self, scores):
        """Add the round's results; plan the next round from `scores` (device tensor of the
        scored job's k-points).  Returns True while a round is left."""
        V = self.system.cell_volume
        for job in self._jobs:
            for k, c in job.calcs.items():
                r = c.result(V, job.nk, job.factor) * job.sign
                self.total[k] = r if k not in self.total else self.total[k] + r
        if self.round >= self.rounds:
            return False
        scored = [j for j in self._jobs if j.scores][0]
        n_top = min(scores.numel(), max(1, int(round(self.top * self.n_grid))))
        sel = np.sort(torch.topk(scores, n_top).indices.cpu().numpy())
        pts = block_points(scored.shifts, scored.fft, 1.0 / np.array(scored.fft) if scored.step is None
                           else scored.step, sel)
        sub_shifts, step = subgrid_shifts(pts, self.cell, self.mesh)
        self.round += 1
        m3 = (self.mesh,) * 3
        self._jobs = [_Job(sub_shifts, m3, step, self._fresh(), self.round < self.rounds, self.mesh ** 3,
                           self.weight, 1.0),
                      _Job(pts, (1, 1, 1), None, self._fresh(), False, 1, self.weight, -1.0)]
        self.kpoints += len(sub_shifts) * self.mesh ** 3 + len(pts)
        self.cell, self.weight = step, self.weight / self.mesh ** 3
        return True

    def result(self):
        return ResultDict(self.total)


def run_refine_omega(system, grid, calculators, precision='mixed', rounds=1, top=0.01, mesh=8, dev_system=None,
                     degen_thresh=1e-4):
    """run() refined around the largest Berry curvatures (OmegaRefinement): `rounds` rounds, each
    refining top x (points of the grid) of the previous round's k-points by mesh^3 sub-grids."""
    engine.require_cuda()
    dev = dev_system or engine.DeviceSystem(system)
    ref = OmegaRefinement(system, grid, calculators, dev.device, rounds, top, mesh)
    while True:
        scores = None
        for job in ref.jobs():
            sc = _evaluate_blocks(dev, system, job.shifts, job.fft, job.step, job.calcs, ref.quantities, precision,
                                  job.scores, degen_thresh, cached_phases=ref.round == 0)
            if job.scores:
                scores = sc
        if not ref.end_round(scores):
            break
    return ref.result()


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
