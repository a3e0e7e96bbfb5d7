"""Drop-in Data_K backend for the reference's own driver.

    import wannierberri as wberri
    from wbgpu.refbind import Data_K_GPU
    wberri.run(system, grid, calculators, data_k_class=Data_K_GPU, ...)
    wberri.run(..., data_k_class=Data_K_GPU, parameters_K={'precision': 'mixed'})

The reference's ``run`` builds one ``Data_K`` per K-point block (run_grid.py:259:
``data_k_class(system, dK=Kp.Kp_fullBZ, grid=grid, Kpoint=Kp, **parameters_K)``), calls every
calculator on it (run_grid.py:260, ``calc(data)``) and sums the returned results times the
K-point factor (run_grid.py:59-66).  ``Data_K_GPU`` subclasses the reference's ``Data_K_R``
(data_K/data_K_R.py:8-22) so that the driver accepts it, and computes nothing on the host:
when a calculator that the GPU serves is called on it, the calculator's GPU twin (the class of
the same name in ``wbgpu.calculators``, built from the same arguments) runs stages 1-4 of that
block on the device -- R->k fields, eigh, U^dagger X U, formula + Fermi scan -- and the result
comes back as the reference's own ``EnergyResult`` (result/energyresult.py:11-90), carrying the
time-reversal and inversion transformations that the reference's formula declares
(calculators/static.py:166-169, calculators/dynamic.py:103-119).  Any other calculator called on
a ``Data_K_GPU`` raises NotImplementedError: there is no CPU fallback.

The system's R-space matrices are uploaded once per reference system object and stay resident
(one ``engine.DeviceSystem`` per system).  Stages 1-3 of a block run once for all its
calculators: the band data are kept on the ``Data_K_GPU`` (grown when a later calculator needs
more fields), which the driver deletes after the block (run_grid.py:261).

Importing this module needs the reference package (``wannierberri``) importable; ``install()``
(called on import) patches the reference's calculator classes once so that their ``__call__``
routes a ``Data_K_GPU`` to the GPU and leaves every other Data_K to the reference's own code.
"""
import weakref

import numpy as np

from wannierberri.data_K.data_K import Data_K
from wannierberri.data_K.data_K_R import Data_K_R
from wannierberri.calculators import static as ref_static
from wannierberri.calculators import dynamic as ref_dynamic
from wannierberri.calculators.calculator import Calculator as RefCalculator
from wannierberri.result import EnergyResult as RefEnergyResult

from . import engine
from . import calculators as gpu_calc
from .system import System_R as GpuSystem

# reference calculator class name -> twin in wbgpu.calculators (same arguments)
STATIC_TWINS = {
    'AHC': 'AHC', 'Morb': 'Morb', 'BerryDipole_FermiSea': 'BerryDipole_FermiSea', 'NLAHC_FermiSea': 'NLAHC_FermiSea',
    'DOS': 'DOS', 'CumDOS': 'CumDOS', 'Ohmic_FermiSea': 'Ohmic_FermiSea', 'Ohmic_FermiSurf': 'Ohmic_FermiSurf',
    'Spin': 'Spin', 'NLDrude_Fermider2': 'NLDrude_Fermider2', 'SHC': 'SHC_static',
    'BerryDipole_FermiSurf': 'BerryDipole_FermiSurf', 'NLAHC_FermiSurf': 'NLAHC_FermiSurf',
    'NLDrude_FermiSurf': 'NLDrude_FermiSurf', 'GME_spin_FermiSurf': 'GME_spin_FermiSurf', 'OmegaOmega': 'OmegaOmega',
    'AHC_Zeeman_spin': 'AHC_Zeeman_spin', 'Hall_classic_FermiSurf': 'Hall_classic_FermiSurf',
    'Hall_classic_FermiSea': 'Hall_classic_FermiSea', 'GME_spin_FermiSea': 'GME_spin_FermiSea',
    'GME_orb_FermiSurf': 'GME_orb_FermiSurf', 'AHC_Zeeman_orb': 'AHC_Zeeman_orb',
}
DYNAMIC_TWINS = {
    'OpticalConductivity': 'OpticalConductivity', 'JDOS': 'JDOS', 'SHC': 'SHC', 'ShiftCurrent': 'ShiftCurrent',
    'InjectionCurrent': 'InjectionCurrent',
}
# R-space keys the device path transforms (engine.KEY_NCOMP plus the Hamiltonian)
DEVICE_KEYS = ('Ham', 'AA', 'BB', 'CC', 'SS', 'SH', 'SA', 'SHA', 'SR', 'SHR')

_SYSTEMS = {}  # id(reference system) -> (weakref, wbgpu System_R, DeviceSystem)


def device_system(system):
    """The wbgpu twin of a reference System_R and its resident device copy, made once per
    system object (R-vectors, lattice, Wannier centres and the R-space matrices the device path
    reads, system/system_R.py:83,106-175)."""
    key = id(system)
    hit = _SYSTEMS.get(key)
    if hit is not None and hit[0]() is system:
        return hit[1], hit[2]
    XX = {k: np.asarray(system.get_R_mat(k)) for k in DEVICE_KEYS if system.has_R_mat(k)}
    gsys = GpuSystem.from_arrays(system.real_lattice, system.rvec.iRvec, system.wannier_centers_cart, XX,
                                 force_internal_terms_only=bool(system.force_internal_terms_only),
                                 periodic=getattr(system, 'periodic', (True, True, True)))
    dev = engine.DeviceSystem(gsys)
    _SYSTEMS[key] = (weakref.ref(system, lambda _r, k=key: _SYSTEMS.pop(k, None)), gsys, dev)
    return gsys, dev


class Data_K_GPU(Data_K_R):
    """One K-point block of the reference's run() evaluated on the GPU (see the module docstring).

    Extra parameter (through ``parameters_K``): ``precision`` -- 'fp64' (default: every stage in
    FP64, the reference's arithmetic) or 'mixed' (double-float eigh, FP32 fields and rotations)."""

    def __init__(self, system, dK=None, grid=None, Kpoint=None, precision='fp64', k_list=None, **parameters):
        if k_list is not None or dK is None:
            raise NotImplementedError("Data_K_GPU evaluates K-point blocks of a Grid (dK); k_list / Path "
                                      "evaluation is not served by the GPU backend")
        if parameters.get('random_gauge'):
            raise NotImplementedError("random_gauge is not supported by the GPU backend")
        if np.isfinite(parameters.get('Emin', -np.inf)) or np.isfinite(parameters.get('Emax', np.inf)):
            raise NotImplementedError("Emin / Emax band selection is not supported by the GPU backend")
        if precision not in ('fp64', 'mixed'):
            raise ValueError(f"precision must be 'fp64' or 'mixed', not {precision!r}")
        # the base bookkeeping of data_K/data_K.py:73-111 only: no FFT plan, no host arrays
        Data_K.__init__(self, system, dK=dK, grid=grid, Kpoint=Kpoint, **parameters)
        self.rvec = None
        self._XX_R = {}
        self.precision = precision
        self._gsys, self._dev = device_system(system)
        self._shift = np.asarray(dK, dtype=float).reshape(1, 3)
        self._NKFFT = tuple(int(n) for n in self.grid.FFT)
        self._bd = None
        self._bd_q = frozenset()

    def band_data(self, quantities, tetra=False):
        """Stages 1-3 of this block on the device, computed once for the union of the fields the
        calculators called so far need."""
        q = frozenset(quantities)
        if self._bd is None or not q <= self._bd_q or (tetra and self._bd.tetra is None):
            q = q | self._bd_q
            corners = None
            if tetra:
                cell = np.asarray(self.Kpoint.dK_fullBZ, dtype=float).reshape(1, 3) / np.array(self._NKFFT)
                corners = engine.BlockCorners(self._dev, self._shift, cell, self._NKFFT, self.precision)
            bd = engine.band_data(self._dev, self._shift, self._NKFFT, set(q), self.precision)
            if corners is not None:
                corners.attach(bd, np.arange(bd.nblocks))
                bd._corners = corners
            self._bd, self._bd_q = bd, q
        return self._bd

    def evaluate(self, twin):
        """The GPU twin's result for this block: histogram / pair sums normalised by the block's
        k-points, K-point factor 1 (what the reference's calculator returns for one Data_K)."""
        bd = self.band_data(twin.quantities(self._gsys), tetra=getattr(twin, 'tetra', False))
        twin.reset(self._dev.device)
        twin.accumulate(bd, self._gsys)
        engine.check_flag(bd)
        corners = getattr(bd, '_corners', None)
        if corners is not None:
            corners.check()
        return twin.result(self._gsys.cell_volume, int(np.prod(self._NKFFT)), 1.0)


# ---------------------------------------------------------------------------------------------
# calculator routing
# ---------------------------------------------------------------------------------------------
_STATIC_ARGS = ('Efermi', 'tetra', 'use_factor', 'kwargs_formula', 'Emin', 'Emax', 'hole_like', 'k_resolved',
                'degen_thresh', 'degen_Kramers', 'save_mode', 'smoother')
_DYNAMIC_ARGS = ('Efermi', 'omega', 'kBT', 'smr_fixed_width', 'smr_type', 'degen_thresh', 'degen_Kramers',
                 'save_mode')


def twin_of(calc):
    """A wbgpu calculator with the reference calculator's class and arguments, or None when the
    GPU serves no such calculator.  The reference instance keeps its constructor arguments as
    attributes (calculators/static.py:26-58, calculators/dynamic.py:28-55) and its final
    constant_factor (after hole_like and the class default)."""
    name = type(calc).__name__
    if isinstance(calc, ref_static.StaticCalculator) and type(calc).__module__ == ref_static.__name__:
        twin_name = STATIC_TWINS.get(name)
        if twin_name is None:
            return None
        kw = {a: getattr(calc, a) for a in _STATIC_ARGS if hasattr(calc, a)}
        kw['kwargs_formula'] = dict(kw.get('kwargs_formula') or {})
        kw['constant_factor'] = calc.constant_factor
        return getattr(gpu_calc, twin_name)(**kw)
    if isinstance(calc, ref_dynamic.DynamicCalculator) and type(calc).__module__ == ref_dynamic.__name__:
        twin_name = DYNAMIC_TWINS.get(name)
        if twin_name is None:
            return None
        kw = {a: getattr(calc, a) for a in _DYNAMIC_ARGS if hasattr(calc, a)}
        kwf = dict(calc.kwargs_formula or {})
        if name == 'SHC':
            kw['SHC_type'] = kwf.pop('SHC_type', 'ryoo')
            kw['shc_abc'] = kwf.pop('shc_abc', None)
        if name == 'ShiftCurrent':
            kw['sc_eta'] = kwf.pop('sc_eta')
        kw['kwargs_formula'] = kwf
        twin = getattr(gpu_calc, twin_name)(**kw)
        twin.constant_factor = calc.constant_factor
        return twin
    return None


# The transformations under time reversal and inversion of each routed calculator's result, as
# the reference's run() returns them (formula objects of formula/covariant.py and
# calculators/dynamic.py:170-360, products by symmetry/point_symmetry.py:486-509).  They are the
# same for every block and every argument set, so they are tabulated here rather than read from a
# formula object, which the reference builds from band data.
_TR_INV = {
    (ref_static, 'AHC'): ('transform_odd', 'transform_ident'),
    (ref_static, 'Morb'): ('transform_odd', 'transform_ident'),
    (ref_static, 'BerryDipole_FermiSea'): ('transform_ident', 'transform_odd'),
    (ref_static, 'NLAHC_FermiSea'): ('transform_ident', 'transform_odd'),
    (ref_static, 'DOS'): ('transform_ident', 'transform_ident'),
    (ref_static, 'CumDOS'): ('transform_ident', 'transform_ident'),
    (ref_static, 'Ohmic_FermiSea'): ('transform_ident', 'transform_ident'),
    (ref_static, 'Ohmic_FermiSurf'): ('transform_ident', 'transform_ident'),
    (ref_static, 'Spin'): ('transform_odd', 'transform_ident'),
    (ref_static, 'NLDrude_Fermider2'): ('transform_odd', 'transform_odd'),
    (ref_static, 'SHC'): ('transform_ident', 'transform_ident'),
    (ref_static, 'BerryDipole_FermiSurf'): ('transform_ident', 'transform_odd'),
    (ref_static, 'NLAHC_FermiSurf'): ('transform_ident', 'transform_odd'),
    (ref_static, 'NLDrude_FermiSurf'): ('transform_odd', 'transform_odd'),
    (ref_static, 'GME_spin_FermiSurf'): ('transform_ident', 'transform_odd'),
    (ref_static, 'OmegaOmega'): ('transform_ident', 'transform_ident'),
    (ref_static, 'AHC_Zeeman_spin'): ('transform_ident', 'transform_ident'),
    (ref_static, 'Hall_classic_FermiSurf'): ('transform_ident', 'transform_ident'),
    (ref_static, 'Hall_classic_FermiSea'): ('transform_ident', 'transform_ident'),
    (ref_static, 'GME_spin_FermiSea'): ('transform_ident', 'transform_odd'),
    (ref_static, 'GME_orb_FermiSurf'): ('transform_ident', 'transform_odd'),
    (ref_static, 'AHC_Zeeman_orb'): ('transform_ident', 'transform_ident'),
    (ref_dynamic, 'OpticalConductivity'): ('transform_trans', 'transform_ident'),
    (ref_dynamic, 'JDOS'): ('transform_ident', 'transform_ident'),
    (ref_dynamic, 'SHC'): ('transform_ident', 'transform_ident'),
    (ref_dynamic, 'ShiftCurrent'): ('transform_ident', 'transform_odd'),
    (ref_dynamic, 'InjectionCurrent'): ('transform_odd_trans_021', 'transform_odd'),
}


def formula_transforms(calc):
    """(transformTR, transformInv) of the reference calculator's result: the reference's own
    Transform objects (symmetry/point_symmetry.py:504-509)."""
    from wannierberri.symmetry import point_symmetry as ps
    mod = ref_static if isinstance(calc, ref_static.StaticCalculator) else ref_dynamic
    tr, inv = _TR_INV[(mod, type(calc).__name__)]
    return getattr(ps, tr), getattr(ps, inv)


def gpu_call(calc, data_K):
    """calc(data_K) for a Data_K_GPU: the twin's block result as the reference's EnergyResult."""
    twin = twin_of(calc)
    if twin is None:
        raise NotImplementedError(f"{type(calc).__module__}.{type(calc).__name__} has no GPU kernel: "
                                  "it cannot be evaluated on a Data_K_GPU (no CPU fallback)")
    tr, inv = formula_transforms(calc)
    res = data_K.evaluate(twin)
    if isinstance(calc, ref_static.StaticCalculator):  # calculators/static.py:166-169
        return RefEnergyResult(calc.Efermi, res.data, transformTR=tr, transformInv=inv,
                               smoothers=[calc.smoother], comment=calc.comment, save_mode=calc.save_mode)
    return RefEnergyResult([calc.Efermi, calc.omega], res.data, transformTR=tr, transformInv=inv,
                           save_mode=calc.save_mode)  # calculators/dynamic.py:116-119


def _all_calculator_classes():
    seen, todo = [], [RefCalculator]
    while todo:
        c = todo.pop()
        for sub in c.__subclasses__():
            if sub not in seen:
                seen.append(sub)
                todo.append(sub)
    return seen


def _route(original):
    def __call__(self, data_K, *a, **k):
        if isinstance(data_K, Data_K_GPU):
            return gpu_call(self, data_K)
        return original(self, data_K, *a, **k)
    __call__._wbgpu_routed = True
    __call__.__wrapped__ = original
    return __call__


def install():
    """Route the reference's calculators: every class that defines its own __call__ (the base
    classes and the overrides below them) gets a wrapper that sends a Data_K_GPU to gpu_call (the
    GPU twin, or NotImplementedError) and any other Data_K to the reference's own method; classes
    that inherit __call__ inherit the wrapper.  Idempotent."""
    for cls in [RefCalculator] + _all_calculator_classes():
        own = cls.__dict__.get('__call__')
        if own is None or getattr(own, '_wbgpu_routed', False):
            continue
        setattr(cls, '__call__', _route(own))


install()
