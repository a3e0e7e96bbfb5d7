"""k-resolved quantities on the GPU path: ``evaluate_k`` and grid tabulation.

Mirrors evaluate_k.py:33-131 (named quantities of evaluate_k.py:9-16) and the Tabulators of
calculators/tabulate.py:21-52: per k-point and band, the trace of the band's degenerate group
(whole band range, no sea group) divided by the group size, for

* ``energy``                          group-averaged E (eV)
* ``band_gradients``                  Re V_nn = dE/dk (eV Angstrom)
* ``berry_curvature``                 Omega (Angstrom^2), internal + external terms
* ``berry_curvature_internal_terms``  internal terms only
* ``berry_curvature_external_terms``  external terms only

Like the reference, a single k-point is a 1x1x1 FFT block with dK = k; a grid tabulates every
block of the grid.  Stages 1-3 are ``engine.band_data`` (FP64 by default), the per-band traces
one ``wbg_berry_tabulate`` launch per term selection.
"""
import ctypes

import numpy as np
import torch

from . import _lib, engine
from .engine import _ptr, _stream

QUANTITIES = ('energy', 'band_gradients', 'berry_curvature', 'berry_curvature_internal_terms',
              'berry_curvature_external_terms')
_TERMS = {'berry_curvature': (1, 1), 'berry_curvature_internal_terms': (1, 0),
          'berry_curvature_external_terms': (0, 1)}


def _check(quantities):
    for q in quantities:
        if q not in QUANTITIES:
            raise ValueError(f"unknown quantity {q}. known quantities are {QUANTITIES}")


def _band_quantities(system, quantities):
    ext = any(_TERMS.get(q, (0, 0))[1] for q in quantities) and not system.force_internal_terms_only
    return {'V', 'A', 'Od'} if ext else {'V'}


def _tab_batch(dev, system, dKs, NKFFT, quantities, precision, degen_thresh, phases=None, block_start=0):
    """Per-k, per-band values of `quantities` for a batch of blocks: dict q -> device tensor."""
    bd = engine.band_data(dev, dKs, NKFFT, _band_quantities(system, quantities), precision, phases=phases,
                          block_start=block_start)
    nkt, nw = bd.nk_total, bd.nw
    lib = _lib.load()
    iA, iO = bd.index.get('A', 0), bd.index.get('Od', 0)

    def terms(q):  # (internal, external) of one quantity's Omega trace
        internal, external = _TERMS.get(q, (1, 0))
        return internal, external if 'A' in bd.index else 0  # no AA_R: internal terms only

    tabs = {}
    for key in {terms(q) for q in quantities}:
        tab = torch.empty((nkt, nw, 7), dtype=torch.float64, device=bd.E.device)
        st = lib.wbg_berry_tabulate(_ptr(bd.E), _ptr(bd.Xbar), bd.Xbar.shape[1], bd.index['V'], iA, iO, nw, nkt,
                                    ctypes.c_double(degen_thresh), key[0], key[1], _ptr(tab), int(bd.fp64_fields),
                                    _stream())
        _lib.check(st, "wbg_berry_tabulate")
        tabs[key] = tab
    engine.check_flag(bd)
    cols = {'energy': slice(0, 1), 'band_gradients': slice(1, 4)}
    out = {}
    for q in quantities:
        t = tabs[terms(q)][:, :, cols.get(q, slice(4, 7))]
        out[q] = t[:, :, 0] if q == 'energy' else t
    return out


def evaluate_k(system, k=(0., 0., 0.), quantities=(), iband=None, return_single_as_dict=False,
               precision='fp64', degen_thresh=1e-4, device='cuda'):
    """evaluate_k.py:33-131 for the named quantities: values at one k-point (reduced
    coordinates) for the bands `iband` (all by default).  Returns {quantity: array}, or the
    array alone for a single quantity unless return_single_as_dict."""
    quantities = list(quantities)
    _check(quantities)
    engine.require_cuda()
    dev = engine.DeviceSystem(system, device)
    res = _tab_batch(dev, system, np.array([k], dtype=float), [1, 1, 1], quantities, precision, degen_thresh)
    if iband is None:
        iband = np.arange(system.num_wann)
    iband = list(np.atleast_1d(iband))
    result = {q: res[q][0].cpu().numpy()[iband] for q in quantities}
    if len(result) == 1 and not return_single_as_dict:
        return next(iter(result.values()))
    return result


def tabulate(system, grid, quantities=('energy', 'berry_curvature'), ibands=None, precision='fp64',
             degen_thresh=1e-4, device='cuda', dev_system=None):
    """Tabulators over every k-point of `grid` (calculators/tabulate.py:21-52): returns
    {'kpoints': (nk, 3) reduced coordinates, quantity: (nk, nbands[, 3])}, k-points block by
    block, each block in C order of its FFT grid."""
    quantities = list(quantities)
    _check(quantities)
    engine.require_cuda()
    dev = dev_system or engine.DeviceSystem(system, device)
    shifts = grid.block_shifts()
    nk = grid.nk_per_block
    from .run import choose_batch
    nb = choose_batch(dev.nw, nk, len(shifts), _band_quantities(system, quantities), precision)
    precs = engine.phase_precs(precision)
    phases = {p: dev.grid_phases(shifts, grid.FFT, p) for p in precs}
    parts = {q: [] for q in quantities}
    for i0 in range(0, len(shifts), nb):
        res = _tab_batch(dev, system, shifts[i0:i0 + nb], grid.FFT, quantities, precision, degen_thresh,
                         phases=phases, block_start=i0)
        for q in quantities:
            parts[q].append(res[q].cpu().numpy())
    sel = slice(None) if ibands is None else list(np.atleast_1d(ibands))
    out = {q: np.concatenate(parts[q])[:, sel] for q in quantities}
    N = np.array(grid.FFT)
    j = np.stack(np.meshgrid(*[np.arange(n) for n in N], indexing='ij'), -1).reshape(-1, 3)
    out['kpoints'] = np.concatenate([j / N + dK for dK in shifts])
    return out
