"""Calculators with the reference's names and arguments, evaluated on the GPU.

Mirrors calculators/static.py:24-169 (StaticCalculator: Fermi-level scan with
cumulative weights, /cell_volume /nk * constant_factor) for ``AHC``
(calculators/static.py:353-364), ``Morb`` (:231-247), ``BerryDipole_FermiSea``
(:472-487), ``DOS`` / ``CumDOS`` (:192-214), ``Ohmic_FermiSea`` / ``Ohmic_FermiSurf``
(:379-403), ``Spin`` (:217-228), and calculators/dynamic.py:26-360 for ``OpticalConductivity``,
``JDOS``, ``SHC``, ``ShiftCurrent`` and ``InjectionCurrent``.  A calculator
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
import types

from .factors import (factor_ahc, factor_morb, factor_ohmic, factor_opt, factor_shc, factor_shift_current,
                      factor_injection_current, factor_nlahc, factor_nldrude, factor_hall_classic, fac_spin_Z,
                      fac_orb_Z, factor_gme_spin, factor_gme_orb)

WBG_FORMULA_IDENTITY, WBG_FORMULA_INVMASS, WBG_FORMULA_VELVEL = 0, 1, 2  # include/wbgpu.h
WBG_FORMULA_OMEGA, WBG_FORMULA_DEROMEGA, WBG_FORMULA_MORB, WBG_FORMULA_DIAG = 3, 4, 5, 6
WBG_FORMULA_VELVELVEL, WBG_FORMULA_SPIN_OMEGA = 7, 8
(WBG_DYN_OPTCOND, WBG_DYN_JDOS, WBG_DYN_SHC_SIMPLE, WBG_DYN_SHC_QIAO, WBG_DYN_SHC_RYOO, WBG_DYN_SHIFT,
 WBG_DYN_INJECTION) = range(7)
from .result import EnergyResult


def fixed_words(n):
    """int64 words of an n-entry fixed-point histogram (the layout of csrc/wbgpu_fixed.cuh)."""
    return 2 * n + 1


def fixed_values(words, n):
    """The n entries of a fixed-point histogram as doubles, rounded exactly as the device does
    (hi 2^4 + ((lo >> 32) 2^-28 + (lo & 2^32-1) 2^-60)); NaN throughout when a contribution
    was not finite."""
    w = np.asarray(words)
    lo = w[0:2 * n:2].view(np.uint64)
    hi = w[1:2 * n:2].astype(np.float64)
    a = (lo & np.uint64(0xffffffff)).astype(np.float64) * 2.0 ** -60
    b = (lo >> np.uint64(32)).astype(np.float64) * 2.0 ** -28
    v = hi * 16.0 + (b + a)
    if w[2 * n] != 0:
        v[:] = np.nan
    return v


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
        # [nEF][ncomp] order-independent fixed-point entries (two int64 words each) and the count
        # of non-finite contributions: the kernels' sums are the same bits whatever the order
        self._hist = torch.zeros(fixed_words(self.nEF_extra * self.ncomp), dtype=torch.int64, device=device)
        if self.tetra:
            self._ef = torch.tensor(self.Efermi, dtype=torch.float64, device=device)

    def tetra_accumulate(self, bd, formula, hist, ncomp, fields, ext=False, product=None):
        """Tetrahedron method for one batch (static.py:80-85,119-125): bands selected by their
        corner energies (sea for fder 0), per-band values of `formula` (or of the in-group
        product `product`, a wbg_product_spec), weighted sum into the histogram in difference
        form (wbg_scan_finalize then yields the result)."""
        tc = bd.tetra
        if tc is None:
            raise RuntimeError("tetra=True needs the corner energies of run() over a regular Grid")
        lib = _lib.load()
        sel = tc.selection(bd, self.Efermi[0], self.Efermi[-1], self.degen_thresh, int(self.fder == 0))
        P = torch.empty((bd.nk_total, bd.nw, ncomp), dtype=torch.float64, device=bd.E.device)
        xbar = _ptr(bd.Xbar) if bd.Xbar is not None else None
        nF = bd.Xbar.shape[1] if bd.Xbar is not None else 0
        if product is not None:
            st = engine._timed('band_values', lib.wbg_product_values, _ptr(bd.E), xbar, nF, ctypes.byref(product),
                               bd.nw, bd.nk_total, ctypes.c_double(self.degen_thresh), _ptr(sel), _ptr(P),
                               int(bd.fp64_fields), _stream())
            _lib.check(st, "wbg_product_values")
        else:
            fi = _lib.FieldIndex(**{k: int(bd.index.get(q, 0)) for k, q in fields.items()})
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
        out = torch.empty((self.nEF_extra, self.ncomp), dtype=torch.float64, device=self._hist.device)
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
                           1 if bd.fp64_fields else engine.MIXED_DEROMEGA_ARITH, _stream())
        _lib.check(st, "wbg_berry_deromega")

    def result(self, cell_volume, nk, factor=1.0):
        data = self.finalize(cell_volume, nk, factor).reshape(-1, 3, 3)
        return EnergyResult(self.Efermi, data.swapaxes(1, 2))


class NLAHC_FermiSea(BerryDipole_FermiSea):
    r"""Nonlinear anomalous Hall conductivity (S^2/A) from the Fermi sea (calculators/static.py:490-498):
    the Berry-curvature dipole times e^3/hbar^2 tau."""

    def __init__(self, constant_factor=factor_nlahc, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)


class SHC_static(StaticCalculator):
    r"""Spin Hall conductivity with dc (S/m) from the Fermi sea (calculators/static.py:647-660, formula
    SpinOmega of formula/covariant.py:759-788): -2 Im(J_nl (D_ln - i A_ln)) / (E_n - E_l) over l outside
    each group, J the spin current of kwargs_formula['spin_current_type'] ('ryoo' default, 'qiao',
    'simple').  Exposed as ``calculators.static.SHC``."""
    ncomp = 27

    def __init__(self, constant_factor=-factor_ahc / 2, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)
        if self.tetra:
            raise NotImplementedError("the static SHC with tetra=True is not supported by the GPU backend")
        self.kind = self.kwargs_formula.get('spin_current_type', 'ryoo')
        kinds = {'simple': WBG_DYN_SHC_SIMPLE, 'qiao': WBG_DYN_SHC_QIAO, 'ryoo': WBG_DYN_SHC_RYOO}
        if self.kind not in kinds:
            raise ValueError(f"spin_current_type must be `qiao` or `ryoo` or `simple`, not {self.kind}")
        self.kind_id = kinds[self.kind]

    def quantities(self, system):
        ext = self.external(system)
        if self.kind != 'simple' and not ext:
            raise NotImplementedError(f"spin Hall {self.kind} without external terms is not implemented yet. "
                                      "Use `SHC_type='simple'`")
        q = {'V', 'S'} | ({'A'} if ext else set())
        if self.kind == 'qiao':
            q |= {'SH', 'SR', 'SHR'}
        elif self.kind == 'ryoo':
            q |= {'SA', 'SHA'}
        return q

    def accumulate(self, bd, system):
        g = lambda q: int(bd.index[q]) if q in bd.index else -1
        spec = _lib.DynamicSpec(formula=self.kind_id, external_terms=int(self.external(system)), V=g('V'), A=g('A'),
                                W=-1, dA=-1, S=g('S'), SH=g('SH'), SA=g('SA'), SHA=g('SHA'), SR=g('SR'), SHR=g('SHR'),
                                sc_eta=0.0, omega_min=0.0, omega_max=0.0)
        sc = self.scan_struct()
        st = engine._timed('berry_scan', _lib.load().wbg_berry_shc, _ptr(bd.E), _ptr(bd.Xbar), bd.Xbar.shape[1],
                           ctypes.byref(spec), bd.nw, bd.nk_total, ctypes.byref(sc), _ptr(self._hist),
                           int(bd.fp64_fields), _stream())
        _lib.check(st, "wbg_berry_shc")

    def result(self, cell_volume, nk, factor=1.0):
        return EnergyResult(self.Efermi, self.finalize(cell_volume, nk, factor).reshape(-1, 3, 3, 3))


class _ScanCalculator(StaticCalculator):
    """Static calculators whose group traces go through wbg_berry_scan (calculators/static.py:60-169):
    Fermi-sea (fder 0) or Fermi-surface (fder 1, central difference over the extended levels)."""
    formula = None
    fields = set()
    field_map = {'V': 'V', 'W': 'W'}  # kernel argument -> band-basis quantity

    def quantities(self, system):
        return set(self.fields)

    def accumulate(self, bd, system):
        if self.tetra:
            return self.tetra_accumulate(bd, self.formula, self._hist, self.ncomp, self.field_map)
        sc = self.scan_struct()
        g = lambda arg: bd.index.get(self.field_map.get(arg), 0)
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
        elif self.fder == 2:  # calculators/static.py:141-142
            data = (data[2:] + data[:-2] - 2 * data[1:-1]) / (self.dEF ** 2)
        return data

    def result(self, cell_volume, nk, factor=1.0):
        data = self._data(cell_volume, nk, factor)
        if self.ncomp == 27:
            data = data.reshape(-1, 3, 3, 3)
        elif self.ncomp == 9:
            data = data.reshape(-1, 3, 3)
        elif self.ncomp == 3:
            data = data.reshape(-1, 3)
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


class NLDrude_Fermider2(_ScanCalculator):
    r"""Drude conductivity (S^2/A) with the second derivative of the distribution
    (calculators/static.py:545-556): -e^3/hbar^2 tau^2 \int [dk] v_b v_a v_c f'' / 2 (formula VelVelVel)."""
    formula, fder, ncomp = WBG_FORMULA_VELVELVEL, 2, 27
    fields = {'V'}

    def __init__(self, constant_factor=factor_nldrude / 2, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)
        if self.tetra:
            raise NotImplementedError("fder=2 with tetra=True is not supported by the GPU backend")


class Spin(_ScanCalculator):
    r"""Spin per unit cell (calculators/static.py:217-228): \int [dk] s f, the Fermi-sea sum of
    Re <n|S|n> (formula Spin, formula/covariant.py:331-335) times the cell volume."""
    formula, fder, ncomp = WBG_FORMULA_DIAG, 0, 3
    fields = {'S'}
    field_map = {'V': 'S'}

    def result(self, cell_volume, nk, factor=1.0):
        data = self._data(cell_volume, nk, factor) * cell_volume
        return EnergyResult(self.Efermi, data.reshape(-1, 3))


class DynamicCalculator(Calculator):
    r"""Kubo-type calculators (calculators/dynamic.py:26-114): every ordered pair of degenerate
    groups at each k-point contributes f_w(E1, E2) (FD(E2) - FD(E1)) M(G1, G2); the result is
    laid out [E_F, omega, components] and scaled by constant_factor / (nk * cell volume).  One
    wbg_dynamic launch pair per chunk of k-points (pair records, then the frequency scan)."""
    formula = None
    real = False  # result dtype float (the reference's dtype=float calculators)
    ndim = 2

    def __init__(self, Efermi=None, omega=None, kBT=0, smr_fixed_width=0.1, smr_type='Lorentzian',
                 kwargs_formula=None, **kwargs):
        super().__init__(**kwargs)
        self.Efermi = np.array(Efermi, dtype=float).reshape(-1)
        self.omega = np.array(omega, dtype=float).reshape(-1)
        self.kBT = kBT
        self.smr_fixed_width = smr_fixed_width
        if smr_type not in ('Lorentzian', 'Gaussian'):
            raise ValueError(f"Invalid smearing type {smr_type}")
        self.smr_type = smr_type
        self.kwargs_formula = dict(kwargs_formula or {})
        self.external_terms = self.kwargs_formula.get('external_terms', True)
        self.sc_eta = 0.0
        self._out = None

    def external(self, system):
        return self.external_terms and not system.force_internal_terms_only

    def formula_id(self):
        return self.formula

    def quantities(self, system):
        return {'V', 'A'} if self.external(system) else {'V'}

    @property
    def ncomp(self):
        return 1 if self.formula == WBG_DYN_JDOS else 9 if self.formula == WBG_DYN_OPTCOND else 27

    def reset(self, device):
        # [E_F][omega][ncomp] complex entries, real and imaginary parts each an order-independent
        # fixed-point entry (csrc/wbgpu_fixed.cuh)
        self._nout = len(self.Efermi) * len(self.omega) * self.ncomp
        self._out = torch.zeros(fixed_words(2 * self._nout), dtype=torch.int64, device=device)
        self._ef = torch.tensor(self.Efermi, dtype=torch.float64, device=device)
        self._om = torch.tensor(self.omega, dtype=torch.float64, device=device)

    def spec(self, bd, system):
        g = lambda q: int(bd.index[q]) if q in bd.index else -1
        return _lib.DynamicSpec(formula=self.formula_id(), external_terms=int(self.external(system)),
                                V=g('V'), A=g('A'), W=g('W'), dA=g('dA'), S=g('S'), SH=g('SH'), SA=g('SA'),
                                SHA=g('SHA'), SR=g('SR'), SHR=g('SHR'), sc_eta=float(self.sc_eta),
                                omega_min=float(self.omega.min()), omega_max=float(self.omega.max()))

    def accumulate(self, bd, system, max_workspace=4 << 30):
        lib = _lib.load()
        kp = _lib.KuboParams(EFmin=float(self.Efermi.min()), EFmax=float(self.Efermi.max()), kBT=float(self.kBT),
                             eta=float(self.smr_fixed_width), degen_thresh=float(self.degen_thresh),
                             nEF=len(self.Efermi), nOmega=len(self.omega), gaussian=int(self.smr_type == 'Gaussian'),
                             reserved=0)
        spec = self.spec(bd, system)
        nw, nkt = bd.nw, bd.nk_total
        per_k = ctypes.c_size_t(0)
        _lib.check(lib.wbg_dynamic_workspace_size(spec.formula, nw, 1, len(self.Efermi), ctypes.byref(per_k)),
                   "wbg_dynamic_workspace_size")
        chunk = max(1, min(nkt, int(max_workspace // per_k.value)))
        ws = ctypes.c_size_t(0)
        _lib.check(lib.wbg_dynamic_workspace_size(spec.formula, nw, chunk, len(self.Efermi), ctypes.byref(ws)),
                   "wbg_dynamic_workspace_size")
        work = torch.empty(int(ws.value), dtype=torch.uint8, device=bd.E.device)
        nF = bd.Xbar.shape[1] if bd.Xbar is not None else 0
        esz = bd.Xbar.element_size() if bd.Xbar is not None else 0
        for k0 in range(0, nkt, chunk):
            n = min(chunk, nkt - k0)
            Xp = ctypes.c_void_p(bd.Xbar.data_ptr() + k0 * nF * nw * nw * esz) if bd.Xbar is not None else None
            Ep = ctypes.c_void_p(bd.E.data_ptr() + k0 * nw * 8)
            st = engine._timed('kubo', lib.wbg_dynamic, Ep, Xp, nF, ctypes.byref(spec), nw, n, ctypes.byref(kp),
                               _ptr(self._ef), _ptr(self._om), _ptr(work), ctypes.c_size_t(work.numel()),
                               _ptr(self._out), int(bd.fp64_fields), _stream())
            _lib.check(st, "wbg_dynamic")

    def select(self, data):
        """[E_F, omega, ncomp] -> the reference's result layout."""
        return data.reshape((len(self.Efermi), len(self.omega)) + (3,) * self.ndim)

    def result(self, cell_volume, nk, factor=1.0):
        v = fixed_values(self._out.cpu().numpy(), 2 * self._nout)
        data = self.select(v[0::2] + 1j * v[1::2])
        data = data * (self.constant_factor / (nk * cell_volume) * factor)
        return EnergyResult([self.Efermi, self.omega], data.real if self.real else data)


class OpticalConductivity(DynamicCalculator):
    r"""Kubo optical conductivity (calculators/dynamic.py:184-196, Formula_OptCond :170-181)."""
    formula = WBG_DYN_OPTCOND

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        self.constant_factor = factor_opt


class JDOS(DynamicCalculator):
    r"""Joint density of states (calculators/dynamic.py:145-162):
    rho(w) = sum_k sum_{m,n} delta(E_m - E_n - w) (f(E_n) - f(E_m)), real."""
    formula, real, ndim = WBG_DYN_JDOS, True, 0

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        self.constant_factor = 1.

    def quantities(self, system):
        return set()


class SHC(DynamicCalculator):
    r"""Spin Hall conductivity (calculators/dynamic.py:199-236): Im(J^{as}_nm (-i A^b_mn)) with the
    spin current J of kind SHC_type ('simple', 'qiao', 'ryoo'; formula/covariant.py:689-756);
    shc_abc = (a, b, c) (1-based) selects one component."""
    ndim = 3

    def __init__(self, SHC_type="ryoo", shc_abc=None, **kwargs):
        super().__init__(**kwargs)
        kinds = {'simple': WBG_DYN_SHC_SIMPLE, 'qiao': WBG_DYN_SHC_QIAO, 'ryoo': WBG_DYN_SHC_RYOO}
        if SHC_type not in kinds:
            raise ValueError(f"spin_current_type must be `qiao` or `ryoo` or `simple`, not {SHC_type}")
        self.SHC_type = SHC_type
        self.formula = kinds[SHC_type]
        if shc_abc is not None:
            assert len(shc_abc) == 3
            self.ndim = 0
        self.shc_abc = shc_abc
        self.constant_factor = factor_shc

    def quantities(self, system):
        ext = self.external(system)
        if self.SHC_type != 'simple' and not ext:
            raise NotImplementedError(f"spin Hall {self.SHC_type} without external terms is not implemented yet. "
                                      "Use `SHC_type='simple'`")
        q = {'V', 'S'} | ({'A'} if ext else set())
        if self.SHC_type == 'qiao':
            q |= {'SH', 'SR', 'SHR'}
        elif self.SHC_type == 'ryoo':
            q |= {'SA', 'SHA'}
        return q

    def select(self, data):
        data = data.reshape(len(self.Efermi), len(self.omega), 3, 3, 3)
        if self.shc_abc is not None:
            a, b, c = (x - 1 for x in self.shc_abc)
            data = data[:, :, a, b, c]
        return data


class ShiftCurrent(DynamicCalculator):
    r"""Shift current (calculators/dynamic.py:302-316, ShiftCurrentFormula :243-299), real;
    sc_eta broadens the principal-value D of the generalised derivative."""
    formula, real, ndim = WBG_DYN_SHIFT, True, 3

    def __init__(self, sc_eta, **kwargs):
        super().__init__(**kwargs)
        self.sc_eta = float(sc_eta)
        self.constant_factor = factor_shift_current

    def quantities(self, system):
        return {'V', 'W', 'A', 'dA'} if self.external(system) else {'V', 'W'}


class InjectionCurrent(DynamicCalculator):
    r"""Injection current (calculators/dynamic.py:346-360, InjectionCurrentFormula :319-343)."""
    formula, ndim = WBG_DYN_INJECTION, 3

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        self.constant_factor = factor_injection_current


# include/wbgpu.h
WBG_FACTOR_VEL, WBG_FACTOR_SPIN, WBG_FACTOR_OMEGA, WBG_FACTOR_MASS, WBG_FACTOR_DERSPIN, WBG_FACTOR_HPLUS = range(6)
_FACTOR_DIM = {WBG_FACTOR_VEL: 3, WBG_FACTOR_SPIN: 3, WBG_FACTOR_OMEGA: 3, WBG_FACTOR_MASS: 9,
               WBG_FACTOR_DERSPIN: 9, WBG_FACTOR_HPLUS: 3}


class _ProductCalculator(StaticCalculator):
    """Static calculators whose formula is an in-group matrix product (formula/formula.py:121-151,
    FormulaProduct; factor lists of formula/covariant.py:798-858) through wbg_berry_product:
    ``factors`` in product order, Fermi surface (fder 1, central difference over the extended
    levels) or Fermi sea (fder 0, the sea group)."""
    factors = ()

    def __init__(self, **kwargs):
        self.ncomp = int(np.prod([_FACTOR_DIM[f] for f in self.factors]))
        super().__init__(**kwargs)

    def quantities(self, system):
        q = set()
        ext = self.external(system)
        for f in self.factors:
            if f == WBG_FACTOR_SPIN:
                q.add('S')
            elif f == WBG_FACTOR_MASS:
                q |= {'V', 'W'}
            elif f == WBG_FACTOR_DERSPIN:
                q |= {'V', 'S', 'dS'}
            else:
                q.add('V')
                if f == WBG_FACTOR_OMEGA and ext:
                    q |= {'A', 'O'}
                if f == WBG_FACTOR_HPLUS and ext:
                    q |= {'A', 'O', 'B', 'C'}
        return q

    def spec(self, bd, system):
        g = lambda q: int(bd.index[q]) if q in bd.index else -1
        fac = list(self.factors) + [0] * (3 - len(self.factors))
        return _lib.ProductSpec(nfactors=len(self.factors), factor=(ctypes.c_int * 3)(*fac),
                                internal_terms=int(self.internal_terms), external_terms=int(self.external(system)),
                                V=g('V'), A=g('A'), O=g('O'), W=g('W'), S=g('S'), B=g('B'), C=g('C'), dS=g('dS'))

    def accumulate(self, bd, system):
        ps = self.spec(bd, system)
        if self.tetra:
            return self.tetra_accumulate(bd, None, self._hist, self.ncomp, None, product=ps)
        sc = self.scan_struct()
        st = engine._timed('berry_product', _lib.load().wbg_berry_product, _ptr(bd.E), _ptr(bd.Xbar),
                           bd.Xbar.shape[1], ctypes.byref(ps), bd.nw, bd.nk_total, ctypes.byref(sc),
                           int(self.fder == 0), _ptr(self._hist), int(bd.fp64_fields), _stream())
        _lib.check(st, "wbg_berry_product")

    def _data(self, cell_volume, nk, factor):
        data = self.finalize(cell_volume, nk, factor)
        if self.fder == 1 and not self.tetra:  # calculators/static.py:137-140
            data = (data[2:] - data[:-2]) / (2 * self.dEF)
        return data.reshape((-1,) + (3,) * sum(1 + (_FACTOR_DIM[f] == 9) for f in self.factors))

    def result(self, cell_volume, nk, factor=1.0):
        return EnergyResult(self.Efermi, self._data(cell_volume, nk, factor))


class BerryDipole_FermiSurf(_ProductCalculator):
    r"""Berry curvature dipole (dimensionless) from the Fermi surface (calculators/static.py:449-458):
    D_bd = -\int [dk] v_b Omega_d f' (formula VelOmega, formula/covariant.py:798-801)."""
    factors, fder = (WBG_FACTOR_VEL, WBG_FACTOR_OMEGA), 1


class NLAHC_FermiSurf(BerryDipole_FermiSurf):
    r"""Nonlinear anomalous Hall conductivity (S^2/A) from the Fermi surface (calculators/static.py:461-469):
    the Fermi-surface Berry-curvature dipole times e^3/hbar^2 tau."""

    def __init__(self, constant_factor=factor_nlahc, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)


class NLDrude_FermiSurf(_ProductCalculator):
    r"""Drude conductivity (S^2/A) from the Fermi surface (calculators/static.py:532-542):
    e^3/hbar^2 tau^2 \int [dk] d_b v_a v_c f' (formula MassVel, formula/covariant.py:830-833)."""
    factors, fder = (WBG_FACTOR_MASS, WBG_FACTOR_VEL), 1

    def __init__(self, constant_factor=factor_nldrude, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)


class GME_spin_FermiSurf(_ProductCalculator):
    r"""Spin gyrotropic magnetoelectric tensor from the Fermi surface (calculators/static.py:340-350):
    \int [dk] v_a s_m f' (formula VelSpin)."""
    factors, fder = (WBG_FACTOR_VEL, WBG_FACTOR_SPIN), 1

    def __init__(self, constant_factor=factor_gme_spin, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)


class OmegaOmega(_ProductCalculator):
    r"""\int [dk] Omega_a Omega_b f' (calculators/static.py:618-623, formula OmegaOmega,
    formula/covariant.py:855-858)."""
    factors, fder = (WBG_FACTOR_OMEGA, WBG_FACTOR_OMEGA), 1


class AHC_Zeeman_spin(_ProductCalculator):
    r"""Spin Zeeman correction of the AHC (S/m/T) from the Fermi surface (calculators/static.py:605-615):
    e^2/hbar \int [dk] Omega_d s_m f' (formula OmegaS, formula/covariant.py:849-852)."""
    factors, fder = (WBG_FACTOR_OMEGA, WBG_FACTOR_SPIN), 1

    def __init__(self, constant_factor=fac_spin_Z * factor_ahc, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)


def _hall_curl(T):
    """The two antisymmetrisations of the classical Hall tensor (calculators/static.py:418-420,
    440-442): T[e, p, q, r, s] -> X[e, p, q, g] = T[.., b(g), a(g)] - T[.., a(g), b(g)], then
    out[e, h, g] = (X[e, a(h), b(h), g] - X[e, b(h), a(h), g]) / 2, (a, b)(g) = (g+1, g+2) mod 3."""
    a, b = [1, 2, 0], [2, 0, 1]
    X = T[:, :, :, b, a] - T[:, :, :, a, b]
    return 0.5 * (X[:, a, b, :] - X[:, b, a, :])


class Hall_classic_FermiSurf(_ProductCalculator):
    r"""Classical Hall conductivity (S/m/T) from the Fermi surface (calculators/static.py:407-424):
    e^3/hbar^2 tau^2 eps_{g m r} \int [dk] v_a d_r v_b v_g f' (formula VelMassVel,
    formula/covariant.py:842-846), antisymmetrised to [E_F, 3, 3]."""
    factors, fder = (WBG_FACTOR_VEL, WBG_FACTOR_MASS, WBG_FACTOR_VEL), 1

    def __init__(self, constant_factor=factor_hall_classic, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)

    def result(self, cell_volume, nk, factor=1.0):
        return EnergyResult(self.Efermi, _hall_curl(self._data(cell_volume, nk, factor)))


class Hall_classic_FermiSea(_ProductCalculator):
    r"""Classical Hall conductivity (S/m/T) from the Fermi sea (calculators/static.py:427-446):
    -e^3/hbar^2 tau^2 eps_{g m r} \int [dk] d_g v_a d_r v_b f (formula MassMass,
    formula/covariant.py:836-839); the second mass tensor's derivative index goes first
    (static.py:438), then the antisymmetrisations of Hall_classic_FermiSurf."""
    factors, fder = (WBG_FACTOR_MASS, WBG_FACTOR_MASS), 0

    def __init__(self, constant_factor=factor_hall_classic, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)

    def result(self, cell_volume, nk, factor=1.0):
        data = self._data(cell_volume, nk, factor).transpose(0, 4, 1, 2, 3)
        return EnergyResult(self.Efermi, _hall_curl(data))


class GME_spin_FermiSea(_ProductCalculator):
    r"""Spin gyrotropic magnetoelectric tensor from the Fermi sea (calculators/static.py:322-337):
    -\int [dk] d_a s_m f (formula DerSpin, the generalised derivative of S, formula/covariant.py:338-342),
    returned with the derivative index first (static.py:334-336)."""
    factors, fder = (WBG_FACTOR_DERSPIN,), 0

    def __init__(self, constant_factor=factor_gme_spin, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)

    def result(self, cell_volume, nk, factor=1.0):
        return EnergyResult(self.Efermi, self._data(cell_volume, nk, factor).swapaxes(1, 2))


class _MinusTwoEfOmega(_ProductCalculator):
    """A product with Morb_Hpm (sign +1) minus 2 E_F times the same product with Omega in its place
    (calculators/static.py:276-281, 639-644): H + G - 2 E_F Omega as the orbital moment."""
    omega_twin = None

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        self._omega = self.omega_twin(**kwargs)

    def quantities(self, system):
        return super().quantities(system) | self._omega.quantities(system)

    def reset(self, device):
        super().reset(device)
        self._omega.reset(device)

    def accumulate(self, bd, system):
        super().accumulate(bd, system)
        self._omega.accumulate(bd, system)

    def result(self, cell_volume, nk, factor=1.0):
        h = self._data(cell_volume, nk, factor)
        om = self._omega._data(cell_volume, nk, factor)
        return EnergyResult(self.Efermi, h - 2.0 * om * self.Efermi.reshape((-1,) + (1,) * (om.ndim - 1)))


class GME_orb_FermiSurf(_MinusTwoEfOmega):
    r"""Orbital gyrotropic magnetoelectric tensor from the Fermi surface (calculators/static.py:266-281):
    \int [dk] v_a m_m f' with m = H + G - 2 E_F Omega (formula VelHplus, formula/covariant.py:804-808,
    minus 2 E_F times BerryDipole_FermiSurf)."""
    factors, fder, omega_twin = (WBG_FACTOR_VEL, WBG_FACTOR_HPLUS), 1, BerryDipole_FermiSurf

    def __init__(self, constant_factor=factor_gme_orb, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)


class AHC_Zeeman_orb(_MinusTwoEfOmega):
    r"""Orbital Zeeman correction of the AHC (S/m/T) from the Fermi surface (calculators/static.py:626-644):
    e^2/hbar \int [dk] Omega_d m_m f' with m = H + G - 2 E_F Omega (formula OmegaHplus,
    formula/covariant.py:861-865, minus 2 E_F times OmegaOmega)."""
    factors, fder, omega_twin = (WBG_FACTOR_OMEGA, WBG_FACTOR_HPLUS), 1, OmegaOmega

    def __init__(self, constant_factor=fac_orb_Z * factor_ahc, **kwargs):
        super().__init__(constant_factor=constant_factor, **kwargs)


# the reference's calculator modules (calculators/static.py, calculators/dynamic.py): both define an SHC
def _no_kernel(name, ref):
    """A calculator of the reference (calculators/static.py) without a GPU kernel here: same name,
    constructing it raises NotImplementedError (there is no CPU fallback)."""
    def __init__(self, *args, **kwargs):
        raise NotImplementedError(f"{name} ({ref}) has no GPU kernel in this backend; there is no CPU fallback")
    return type(name, (StaticCalculator,), {'__init__': __init__, '__doc__': f"Not available: {ref}."})


_NO_KERNEL = {
    'NLDrude_FermiSea': 'calculators/static.py:519-529', 'GME_orb_FermiSea': 'calculators/static.py:284-300',
    'eMChA_FermiSurf': 'calculators/static.py:560-565', 'NLDrude_Zeeman_spin': 'calculators/static.py:568-573',
    'NLDrude_Zeeman_orb_Omega': 'calculators/static.py:576-581', 'NLDrude_Zeeman_orb': 'calculators/static.py:584-600',
    'QuantumMetric_FermiSea': 'calculators/static.py:663-670', 'QuantumMetric_Vel_DQ': 'calculators/static.py:673-680'}
_no_kernel_classes = {n: _no_kernel(n, r) for n, r in _NO_KERNEL.items()}
globals().update(_no_kernel_classes)

static = types.SimpleNamespace(**_no_kernel_classes, **dict(
    StaticCalculator=StaticCalculator, AHC=AHC, Morb=Morb, BerryDipole_FermiSea=BerryDipole_FermiSea,
    NLAHC_FermiSea=NLAHC_FermiSea, DOS=DOS, CumDOS=CumDOS, Ohmic_FermiSea=Ohmic_FermiSea,
    Ohmic_FermiSurf=Ohmic_FermiSurf, Spin=Spin, NLDrude_Fermider2=NLDrude_Fermider2, SHC=SHC_static,
    BerryDipole_FermiSurf=BerryDipole_FermiSurf, NLAHC_FermiSurf=NLAHC_FermiSurf, NLDrude_FermiSurf=NLDrude_FermiSurf,
    GME_spin_FermiSurf=GME_spin_FermiSurf, OmegaOmega=OmegaOmega, AHC_Zeeman_spin=AHC_Zeeman_spin,
    Hall_classic_FermiSurf=Hall_classic_FermiSurf, Hall_classic_FermiSea=Hall_classic_FermiSea,
    GME_spin_FermiSea=GME_spin_FermiSea, GME_orb_FermiSurf=GME_orb_FermiSurf, AHC_Zeeman_orb=AHC_Zeeman_orb))
def _elsewhere(name, ref, hint):
    """A calculator class of the reference served differently here (or not at all): constructing it
    raises NotImplementedError that says where the equivalent lives."""
    def __init__(self, *args, **kwargs):
        raise NotImplementedError(f"{name} ({ref}): {hint}")
    return type(name, (Calculator,), {'__init__': __init__, '__doc__': f"Not available as a calculator: {ref}."})


_TAB_HINT = ("tabulation runs through wbgpu.tabulate(system, grid, quantities) (energy, band_gradients, "
             "berry_curvature and its terms) and wbgpu.evaluate_k, not as a run() calculator")
tabulate = types.SimpleNamespace(**{n: _elsewhere(n, f'calculators/tabulate.py:{r}', _TAB_HINT) for n, r in {
    'Tabulator': '12-53', 'TabulatorAll': '56-119', 'Energy': '122-125', 'Velocity': '128-131', 'InvMass': '134-138',
    'Der3E': '141-145', 'BerryCurvature': '148-152', 'DerBerryCurvature': '155-159', 'Der2BerryCurvature': '162-166',
    'Spin': '169-173', 'DerSpin': '176-180', 'Der2Spin': '183-186', 'OrbitalMoment': '189-193',
    'DerOrbitalMoment': '196-200', 'Der2OrbitalMoment': '210-215', 'SpinBerry': '218-221'}.items()})
sdct = types.SimpleNamespace(**{n: _elsewhere(n, f'calculators/sdct.py:{r}', "the spatially dispersive "
                                              "conductivity has no GPU kernel in this backend; no CPU fallback exists")
                                for n, r in {'SDCT_asym': '37-40', 'SDCT_sym': '43-46', 'SDCT_sym_sea_I': '77-84',
                                             'SDCT_asym_sea_I': '87-94', 'SDCT_sym_sea_II': '97-104',
                                             'SDCT_asym_sea_II': '107-114', 'SDCT_sym_surf_I': '123-130',
                                             'SDCT_asym_surf_I': '133-140', 'SDCT_sym_surf_II': '143-150',
                                             'SDCT_asym_surf_II': '153-160'}.items()})
TabulatorAll = tabulate.TabulatorAll

dynamic = types.SimpleNamespace(
    DynamicCalculator=DynamicCalculator, OpticalConductivity=OpticalConductivity, JDOS=JDOS, SHC=SHC,
    ShiftCurrent=ShiftCurrent, InjectionCurrent=InjectionCurrent)
