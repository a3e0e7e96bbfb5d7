"""Calculators with the reference's names and arguments, evaluated on the GPU.

Mirrors calculators/static.py:24-169 (StaticCalculator: Fermi-level scan with
cumulative weights, /cell_volume /nk * constant_factor) for ``AHC``
(calculators/static.py:353-364).  A calculator declares the band-basis quantities it
needs (``quantities``), accumulates a device histogram per batch of blocks
(``accumulate``) and turns it into an ``EnergyResult`` (``finalize``).  Formulae
without a GPU kernel raise NotImplementedError: there is no CPU fallback.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from . import engine
from .engine import _ptr, _stream
from .factors import factor_ahc
from .result import EnergyResult


class Calculator:
    def __init__(self, degen_thresh=1e-4, degen_Kramers=False, save_mode="bin+txt", print_comment=False):
        if degen_Kramers:
            raise NotImplementedError("degen_Kramers is not supported by the GPU backend")
        self.degen_thresh = degen_thresh
        self.save_mode = save_mode


class StaticCalculator(Calculator):
    fder = 0
    ncomp = 3

    def __init__(self, Efermi, tetra=False, smoother=None, constant_factor=1., use_factor=True,
                 kwargs_formula=None, Emin=-np.inf, Emax=np.inf, hole_like=False, k_resolved=False, **kwargs):
        super().__init__(**kwargs)
        if tetra or k_resolved or hole_like or smoother is not None:
            raise NotImplementedError("tetra / k_resolved / hole_like / smoother are not supported by the GPU backend")
        self.Efermi = np.array(Efermi, dtype=float)
        self.constant_factor = constant_factor
        self.use_factor = use_factor
        self.kwargs_formula = dict(kwargs_formula or {})
        self.internal_terms = self.kwargs_formula.get('internal_terms', True)
        self.external_terms = self.kwargs_formula.get('external_terms', True)
        # calculators/static.py:53-58
        self.extraEf = 0 if self.fder == 0 else 1 if self.fder in (1, 2) else 2
        self.dEF = self.Efermi[1] - self.Efermi[0] if len(self.Efermi) > 1 else 0.001
        self.EFmin = self.Efermi[0] - self.extraEf * self.dEF
        self.EFmax = self.Efermi[-1] + self.extraEf * self.dEF
        self.nEF_extra = self.Efermi.shape[0] + 2 * self.extraEf
        self._hist = None

    def scan_struct(self):
        return _lib.Scan(EFmin=float(self.EFmin), EFmax=float(self.EFmax), dEF=float(self.dEF),
                         degen_thresh=float(self.degen_thresh), nEF=int(self.nEF_extra), reserved=0)

    def external(self, system):
        return self.external_terms and not system.force_internal_terms_only

    def reset(self, device):
        self._hist = torch.zeros((self.nEF_extra, self.ncomp), dtype=torch.float64, device=device)

    def finalize(self, cell_volume, nk, factor=1.0):
        """Cumulative scan and normalisation (static.py:127-155) times the K-point factor."""
        cf = self.constant_factor if self.use_factor else np.sign(self.constant_factor)
        scale = cf / (cell_volume * nk) * factor
        out = torch.empty_like(self._hist)
        _lib.check(_lib.load().wbg_scan_finalize(_ptr(self._hist), self.nEF_extra, self.ncomp, ctypes.c_double(scale),
                                                 _ptr(out), _stream()), "wbg_scan_finalize")
        return out.cpu().numpy()


class AHC(StaticCalculator):
    r"""Anomalous Hall conductivity (S/m): O = -e^2/hbar \int [dk] Omega f (calculators/static.py:353-364)."""

    def __init__(self, constant_factor=factor_ahc, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)

    def quantities(self, system):
        return {'V', 'A', 'O'} if self.external(system) else {'V'}

    def accumulate(self, bd, system):
        ext = self.external(system)
        sc = self.scan_struct()
        iA = bd.index.get('A', 0)
        iO = bd.index.get('O', 0)
        st = engine._timed('berry_omega', _lib.load().wbg_berry_omega, _ptr(bd.E), _ptr(bd.Xbar), bd.Xbar.shape[1], bd.index['V'], iA, iO, bd.nw,
                                         bd.nk_total, ctypes.byref(sc), int(self.internal_terms), int(ext),
                                         _ptr(self._hist), int(bd.fp64_fields), _stream())
        _lib.check(st, "wbg_berry_omega")

    def result(self, cell_volume, nk, factor=1.0):
        return EnergyResult(self.Efermi, self.finalize(cell_volume, nk, factor))
