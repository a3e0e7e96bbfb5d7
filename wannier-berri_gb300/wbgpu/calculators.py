"""Calculators with the reference's names and arguments, evaluated on the GPU.

Mirrors calculators/static.py:24-169 (StaticCalculator: Fermi-level scan with
cumulative weights, /cell_volume /nk * constant_factor) for ``AHC``
(calculators/static.py:353-364), ``Morb`` (:231-247), ``BerryDipole_FermiSea``
(:472-487), ``DOS`` / ``CumDOS`` (:192-214), ``Ohmic_FermiSea`` / ``Ohmic_FermiSurf``
(:379-403), and calculators/dynamic.py:26-196 for ``OpticalConductivity``.  A calculator
declares the band-basis quantities it needs (``quantities``), accumulates a device histogram
per batch of blocks (``accumulate``) and turns it into an ``EnergyResult`` (``finalize``).
With ``tetra=True`` the static calculators use the tetrahedron method (static.py:80-125,
grid/tetrahedron.py): per-band values (wbg_band_values) weighted by the tetrahedron
occupations of the corner energies (wbg_tetra_accumulate).  Formulae without a GPU kernel
raise NotImplementedError: there is no CPU fallback.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from . import engine
from .engine import _ptr, _stream
from .factors import factor_ahc, factor_morb, factor_ohmic, factor_opt

WBG_FORMULA_IDENTITY, WBG_FORMULA_INVMASS, WBG_FORMULA_VELVEL = 0, 1, 2  # include/wbgpu.h
WBG_FORMULA_OMEGA, WBG_FORMULA_DEROMEGA, WBG_FORMULA_MORB = 3, 4, 5
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
        if k_resolved or hole_like or smoother is not None:
            raise NotImplementedError("k_resolved / hole_like / smoother are not supported by the GPU backend")
        if tetra and np.isfinite(Emin):
            raise NotImplementedError("tetra=True with a finite Emin is not supported by the GPU backend")
        self.tetra = bool(tetra)
        self.Efermi = np.array(Efermi, dtype=float)
        self.constant_factor = constant_factor
        self.use_factor = use_factor
        self.kwargs_formula = dict(kwargs_formula or {})
        self.internal_terms = self.kwargs_formula.get('internal_terms', True)
        self.external_terms = self.kwargs_formula.get('external_terms', True)
        # calculators/static.py:53-58 (the tetrahedron weights need no extra levels)
        self.extraEf = 0 if (self.fder == 0 or self.tetra) else 1 if self.fder in (1, 2) else 2
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
        if self.tetra:
            self._ef = torch.tensor(self.Efermi, dtype=torch.float64, device=device)

    def tetra_accumulate(self, bd, formula, hist, ncomp, fields, ext=False):
        """Tetrahedron method for one batch (static.py:80-85,119-125): bands selected by their
        corner energies (sea for fder 0), per-band values of `formula`, weighted sum into the
        histogram in difference form (wbg_scan_finalize then yields the result)."""
        tc = bd.tetra
        if tc is None:
            raise RuntimeError("tetra=True needs the corner energies of run() over a regular Grid")
        lib = _lib.load()
        sel = tc.selection(bd, self.Efermi[0], self.Efermi[-1], self.degen_thresh, int(self.fder == 0))
        P = torch.empty((bd.nk_total, bd.nw, ncomp), dtype=torch.float64, device=bd.E.device)
        fi = _lib.FieldIndex(**{k: int(bd.index.get(q, 0)) for k, q in fields.items()})
        xbar = _ptr(bd.Xbar) if bd.Xbar is not None else None
        nF = bd.Xbar.shape[1] if bd.Xbar is not None else 0
        st = engine._timed('band_values', lib.wbg_band_values, _ptr(bd.E), xbar, nF, ctypes.byref(fi), bd.nw,
                           bd.nk_total, formula, int(self.internal_terms), int(ext),
                           ctypes.c_double(self.degen_thresh), _ptr(sel), _ptr(P), int(bd.fp64_fields), _stream())
        _lib.check(st, "wbg_band_values")
        ascending = int(len(self.Efermi) < 2 or np.all(np.diff(self.Efermi) > 0))
        st = engine._timed('tetra_accumulate', lib.wbg_tetra_accumulate, _ptr(bd.E), _ptr(tc.Ec), _ptr(tc.slot),
                           _ptr(bd.tetra_blocks), bd.nblocks, ctypes.byref(tc.grid), bd.nw, _ptr(sel), _ptr(P), ncomp,
                           _ptr(self._ef), len(self.Efermi), int(self.fder), ascending, int(bd.fp64_fields),
                           _ptr(hist), _stream())
        _lib.check(st, "wbg_tetra_accumulate")

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
        return {'V', 'A', 'Od'} if self.external(system) else {'V'}

    def accumulate(self, bd, system):
        ext = self.external(system)
        if self.tetra:
            return self.tetra_accumulate(bd, WBG_FORMULA_OMEGA, self._hist, 3, {'V': 'V', 'A': 'A', 'O': 'Od'}, ext)
        sc = self.scan_struct()
        iA = bd.index.get('A', 0)
        iO = bd.index.get('Od', 0)
        st = engine._timed('berry_omega', _lib.load().wbg_berry_omega, _ptr(bd.E), _ptr(bd.Xbar), bd.Xbar.shape[1], bd.index['V'], iA, iO, bd.nw,
                                         bd.nk_total, ctypes.byref(sc), int(self.internal_terms), int(ext),
                                         _ptr(self._hist), bd.omega_mode, _stream())
        _lib.check(st, "wbg_berry_omega")

    def result(self, cell_volume, nk, factor=1.0):
        return EnergyResult(self.Efermi, self.finalize(cell_volume, nk, factor))


class Morb(StaticCalculator):
    r"""Orbital magnetic moment per unit cell (mu_B): M = -\int [dk] (H + G - 2 E_f Omega) f
    (calculators/static.py:231-247; formula Morb_Hpm, formula/covariant.py:424-449)."""

    def __init__(self, constant_factor=factor_morb, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)

    def quantities(self, system):
        return {'V', 'A', 'Od', 'B', 'C'} if self.external(system) else {'V'}

    def reset(self, device):
        super().reset(device)
        self._hist_omega = torch.zeros_like(self._hist)

    def accumulate(self, bd, system):
        ext = self.external(system)
        if self.tetra:
            f = {'V': 'V', 'A': 'A', 'O': 'Od', 'B': 'B', 'C': 'C'}
            self.tetra_accumulate(bd, WBG_FORMULA_MORB, self._hist, 3, f, ext)
            return self.tetra_accumulate(bd, WBG_FORMULA_OMEGA, self._hist_omega, 3, f, ext)
        sc = self.scan_struct()
        lib = _lib.load()
        g = lambda q: bd.index.get(q, 0)
        st = engine._timed('berry_morb', lib.wbg_berry_morb, _ptr(bd.E), _ptr(bd.Xbar), bd.Xbar.shape[1], g('V'),
                           g('A'), g('Od'), g('B'), g('C'), bd.nw, bd.nk_total, ctypes.byref(sc),
                           int(self.internal_terms), int(ext), _ptr(self._hist), int(bd.fp64_fields), _stream())
        _lib.check(st, "wbg_berry_morb")
        st = engine._timed('berry_omega', lib.wbg_berry_omega, _ptr(bd.E), _ptr(bd.Xbar), bd.Xbar.shape[1],
                           g('V'), g('A'), g('Od'), bd.nw, bd.nk_total, ctypes.byref(sc), int(self.internal_terms),
                           int(ext), _ptr(self._hist_omega), bd.omega_mode, _stream())
        _lib.check(st, "wbg_berry_omega")

    def result(self, cell_volume, nk, factor=1.0):
        H = self.finalize(cell_volume, nk, factor)
        hist = self._hist
        self._hist = self._hist_omega
        O = self.finalize(cell_volume, nk, factor)
        self._hist = hist
        return EnergyResult(self.Efermi, (H - 2.0 * self.Efermi[:, None] * O) * cell_volume)


class BerryDipole_FermiSea(StaticCalculator):
    r"""Berry curvature dipole (dimensionless): D = \int [dk] d_b Omega_d f
    (calculators/static.py:472-487; formula DerOmega, formula/covariant.py:212-259)."""
    ncomp = 9

    def quantities(self, system):
        return {'V', 'W', 'A', 'O', 'dA', 'dO'} if self.external(system) else {'V', 'W'}

    def accumulate(self, bd, system):
        ext = self.external(system)
        if self.tetra:
            f = {'V': 'V', 'A': 'A', 'O': 'O', 'W': 'W', 'dA': 'dA', 'dO': 'dO'}
            return self.tetra_accumulate(bd, WBG_FORMULA_DEROMEGA, self._hist, 9, f, ext)
        sc = self.scan_struct()
        g = lambda q: bd.index.get(q, 0)
        st = engine._timed('berry_deromega', _lib.load().wbg_berry_deromega, _ptr(bd.E), _ptr(bd.Xbar),
                           bd.Xbar.shape[1], g('V'), g('A'), g('O'), g('W'), g('dA'), g('dO'), bd.nw, bd.nk_total,
                           ctypes.byref(sc), int(self.internal_terms), int(ext), _ptr(self._hist),
                           int(bd.fp64_fields), _stream())
        _lib.check(st, "wbg_berry_deromega")

    def result(self, cell_volume, nk, factor=1.0):
        data = self.finalize(cell_volume, nk, factor).reshape(-1, 3, 3)
        return EnergyResult(self.Efermi, data.swapaxes(1, 2))


class _ScanCalculator(StaticCalculator):
    """Static calculators whose group traces go through wbg_berry_scan (calculators/static.py:60-169):
    Fermi-sea (fder 0) or Fermi-surface (fder 1, central difference over the extended levels)."""
    formula = None
    fields = set()

    def quantities(self, system):
        return set(self.fields)

    def accumulate(self, bd, system):
        if self.tetra:
            return self.tetra_accumulate(bd, self.formula, self._hist, self.ncomp, {'V': 'V', 'W': 'W'})
        sc = self.scan_struct()
        g = lambda q: bd.index.get(q, 0)
        xbar = _ptr(bd.Xbar) if bd.Xbar is not None else None
        nF = bd.Xbar.shape[1] if bd.Xbar is not None else 0
        st = engine._timed('berry_scan', _lib.load().wbg_berry_scan, _ptr(bd.E), xbar, nF, g('V'), g('W'), bd.nw,
                           bd.nk_total, ctypes.byref(sc), self.formula, int(self.fder == 0), _ptr(self._hist),
                           int(bd.fp64_fields), _stream())
        _lib.check(st, "wbg_berry_scan")

    def _data(self, cell_volume, nk, factor):
        data = self.finalize(cell_volume, nk, factor)
        if self.fder == 1 and not self.tetra:  # calculators/static.py:137-140
            data = (data[2:] - data[:-2]) / (2 * self.dEF)
        return data

    def result(self, cell_volume, nk, factor=1.0):
        data = self._data(cell_volume, nk, factor)
        if self.ncomp == 9:
            data = data.reshape(-1, 3, 3)
        else:
            data = data.reshape(-1)
        return EnergyResult(self.Efermi, data)


class CumDOS(_ScanCalculator):
    r"""Cumulative density of states (calculators/static.py:192-214): states per cell below E_F."""
    formula, fder, ncomp = WBG_FORMULA_IDENTITY, 0, 1

    def result(self, cell_volume, nk, factor=1.0):
        data = self._data(cell_volume, nk, factor) * cell_volume  # _DOS.__call__ (static.py:198-200)
        return EnergyResult(self.Efermi, data.reshape(-1))


class DOS(CumDOS):
    r"""Density of states (calculators/static.py:203-207): states per cell per eV."""
    fder = 1


class Ohmic_FermiSea(_ScanCalculator):
    r"""Ohmic conductivity (S/m, tau = 1 fs) from the Fermi sea (calculators/static.py:379-390):
    sigma_ab = e^2/hbar tau \int [dk] d_b v_a f (formula InvMass)."""
    formula, fder, ncomp = WBG_FORMULA_INVMASS, 0, 9
    fields = {'V', 'W'}

    def __init__(self, constant_factor=factor_ohmic, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)


class Ohmic_FermiSurf(_ScanCalculator):
    r"""Ohmic conductivity (S/m, tau = 1 fs) from the Fermi surface (calculators/static.py:393-403):
    sigma_ab = -e^2/hbar tau \int [dk] v_a v_b f' (formula VelVel)."""
    formula, fder, ncomp = WBG_FORMULA_VELVEL, 1, 9
    fields = {'V'}

    def __init__(self, constant_factor=factor_ohmic, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)


class OpticalConductivity(Calculator):
    r"""Kubo optical conductivity (calculators/dynamic.py:184-196, Formula_OptCond :170-181)."""

    def __init__(self, Efermi=None, omega=None, kBT=0, smr_fixed_width=0.1, smr_type='Lorentzian',
                 kwargs_formula=None, **kwargs):
        super().__init__(**kwargs)
        self.Efermi = np.array(Efermi, dtype=float).reshape(-1)
        self.omega = np.array(omega, dtype=float)
        self.kBT = kBT
        self.smr_fixed_width = smr_fixed_width
        if smr_type not in ('Lorentzian', 'Gaussian'):
            raise ValueError(f"Invalid smearing type {smr_type}")
        self.smr_type = smr_type
        self.kwargs_formula = dict(kwargs_formula or {})
        self.external_terms = self.kwargs_formula.get('external_terms', True)
        self.constant_factor = factor_opt
        self._out = None

    def external(self, system):
        return self.external_terms and not system.force_internal_terms_only

    def quantities(self, system):
        return {'V', 'A'} if self.external(system) else {'V'}

    def reset(self, device):
        self._out = torch.zeros((len(self.Efermi), len(self.omega), 9), dtype=torch.complex128, device=device)
        self._ef = torch.tensor(self.Efermi, dtype=torch.float64, device=device)
        self._om = torch.tensor(self.omega, dtype=torch.float64, device=device)

    def accumulate(self, bd, system, max_workspace=4 << 30):
        lib = _lib.load()
        ext = self.external(system)
        kp = _lib.KuboParams(EFmin=float(self.Efermi.min()), EFmax=float(self.Efermi.max()), kBT=float(self.kBT),
                             eta=float(self.smr_fixed_width), degen_thresh=float(self.degen_thresh),
                             nEF=len(self.Efermi), nOmega=len(self.omega), gaussian=int(self.smr_type == 'Gaussian'),
                             reserved=0)
        nw, nkt = bd.nw, bd.nk_total
        per_k = ctypes.c_size_t(0)
        _lib.check(lib.wbg_kubo_workspace_size(nw, 1, len(self.Efermi), ctypes.byref(per_k)), "wbg_kubo_workspace_size")
        chunk = max(1, min(nkt, int(max_workspace // per_k.value)))
        ws = ctypes.c_size_t(0)
        _lib.check(lib.wbg_kubo_workspace_size(nw, chunk, len(self.Efermi), ctypes.byref(ws)), "wbg_kubo_workspace_size")
        work = torch.empty(int(ws.value), dtype=torch.uint8, device=bd.E.device)
        nF = bd.Xbar.shape[1]
        esz = bd.Xbar.element_size()
        for k0 in range(0, nkt, chunk):
            n = min(chunk, nkt - k0)
            Xp = ctypes.c_void_p(bd.Xbar.data_ptr() + k0 * nF * nw * nw * esz)
            Ep = ctypes.c_void_p(bd.E.data_ptr() + k0 * nw * 8)
            st = engine._timed('kubo', lib.wbg_kubo, Ep, Xp, nF, bd.index['V'], bd.index.get('A', 0), nw, n, int(ext),
                               ctypes.byref(kp), _ptr(self._ef), _ptr(self._om), _ptr(work),
                               ctypes.c_size_t(work.numel()), _ptr(self._out), int(bd.fp64_fields), _stream())
            _lib.check(st, "wbg_kubo")

    def result(self, cell_volume, nk, factor=1.0):
        data = self._out.cpu().numpy().reshape(len(self.Efermi), len(self.omega), 3, 3)
        data = data * (self.constant_factor / (nk * cell_volume) * factor)
        return EnergyResult([self.Efermi, self.omega], data)
