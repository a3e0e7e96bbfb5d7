"""GPU parity of the dynamic calculators (JDOS, SHC, shift and injection currents) and of the static
Spin, SHC (SpinOmega), NLDrude_Fermider2 and NLAHC_FermiSea, through wbgpu.run (C ABI: wbg_dynamic,
wbg_berry_scan with WBG_FORMULA_DIAG / WBG_FORMULA_VELVELVEL, wbg_berry_shc).

* the reference's own stored results of tests/test_run.py:653-669 on its random system
  (random-spin, random-opt_SHCqiao, random-opt_SHCryoo);
* dynamic_ref.npz: the reference's run() on the same system for every dynamic formula
  (tests/golden/make_golden.py, section 7);
* static_ref.npz: the reference's run() for the static SHC, NLDrude_Fermider2, NLAHC_FermiSea
  (section 8);
* the oracle on the triclinic MDRS model (nw = 6, anisotropic FFT grid) for the formulas that need
  no spin matrices, FP64 and mixed precision.
Pair records and the frequency scan are FP64 in the FP64 path and FP32 (with FP64 energy differences)
in the mixed path: FP64 path within 1e-8 of max|ref| (the reference goldens' rule), mixed path within
1e-6.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import wb_oracle as O  # noqa: E402
from wbgpu import models, system as wsys  # noqa: E402
import wbgpu  # noqa: E402

C = wbgpu.calculators


def _random_system(golden_dir):
    f = np.load(os.path.join(golden_dir, 'random_system.npz'))
    XX = {k[5:]: f[k] for k in f.files if k.startswith('XX_R_')}
    return wsys.System_R.from_arrays(f['real_lattice'], f['iRvec'], f['wannier_centers_cart'], XX)


def _close(got, ref, tol):
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) <= tol * np.max(np.abs(ref)), np.max(np.abs(got - ref)) / np.max(np.abs(ref))


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-8), ('mixed', 1e-6)])
def test_spin_shc_reference_golden(golden_dir, precision, tol):
    """random-spin, random-opt_SHCqiao, random-opt_SHCryoo (tests/test_run.py:653-669: NK 6 = 2 x 3,
    SHC at E_F 17, 18 eV, omega 0..7 eV, Gaussian 0.2 eV)."""
    s = _random_system(golden_dir)
    ref = np.load(os.path.join(golden_dir, 'random_results.npz'))
    popt = dict(Efermi=np.array([17.0, 18.0]), omega=np.arange(0.0, 7.1, 1.0), smr_fixed_width=0.20,
                smr_type="Gaussian")
    calcs = {'spin': C.Spin(Efermi=np.linspace(-2, 2, 5)), 'opt_SHCqiao': C.SHC(SHC_type="qiao", **popt),
             'opt_SHCryoo': C.SHC(SHC_type="ryoo", **popt)}
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=3), calcs, precision=precision)
    _close(res['spin'].data, ref['spin_data'], 1e-8 if precision == 'fp64' else tol)
    for q in ('opt_SHCqiao', 'opt_SHCryoo'):
        _close(res[q].data, ref[q + '_data'], tol)


def _dynamic_gpu_calculators(EF, om):
    pL = dict(Efermi=EF, omega=om, smr_fixed_width=0.3)
    pG = dict(Efermi=EF, omega=om, smr_fixed_width=0.2, smr_type='Gaussian', kBT=0.05)
    return {'jdos_L': C.JDOS(**pL), 'jdos_G': C.JDOS(**pG),
            'shc_simple_L': C.SHC(SHC_type='simple', **pL),
            'shc_simple_int_G': C.SHC(SHC_type='simple', kwargs_formula={'external_terms': False}, **pG),
            'shc_qiao_L': C.SHC(SHC_type='qiao', **pL), 'shc_ryoo_G': C.SHC(SHC_type='ryoo', **pG),
            'shc_ryoo_abc_L': C.SHC(SHC_type='ryoo', shc_abc=(1, 2, 3), **pL),
            'shift_G': C.ShiftCurrent(sc_eta=0.1, **pG),
            'shift_int_L': C.ShiftCurrent(sc_eta=0.1, kwargs_formula={'external_terms': False}, **pL),
            'injection_G': C.InjectionCurrent(**pG), 'injection_L': C.InjectionCurrent(**pL),
            'spin': C.Spin(Efermi=np.linspace(-3, 3, 11))}


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-8), ('mixed', 1e-6)])
def test_dynamic_reference_run(golden_dir, precision, tol):
    """Every dynamic formula against the reference's run() on the random system (dynamic_ref.npz)."""
    s = _random_system(golden_dir)
    ref = np.load(os.path.join(golden_dir, 'dynamic_ref.npz'))
    calcs = _dynamic_gpu_calculators(ref['EF'], ref['omega'])
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=3), calcs, precision=precision)
    for q in calcs:
        r = ref['random_' + q]
        assert res[q].data.dtype.kind == r.dtype.kind, q
        _close(res[q].data, r, 1e-8 if (q == 'spin' and precision == 'fp64') else tol)


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-8), ('mixed', 1e-6)])
def test_dynamic_mdrs_vs_oracle(precision, tol):
    """JDOS, shift and injection currents on the triclinic MDRS model (anisotropic FFT grid) against
    the oracle: exercises Hermitian-base fields (lower triangles in the mixed path), W and dA."""
    d = models.config_system(2, small=True)
    s = wsys.System_R.from_dict(d)
    s.do_ws_dist(3)
    o = O.RSystem(s.real_lattice, s.iRvec, s.wannier_centers_cart, s._XX_R)
    EF = np.array([-0.5, 0.0, 0.4])
    om = np.linspace(0.05, 2.0, 9)
    p = dict(Efermi=EF, omega=om, smr_fixed_width=0.15)
    mk = lambda M: {'jdos': M.JDOS(**p), 'shift': M.ShiftCurrent(sc_eta=0.05, **p),
                    'inj': M.InjectionCurrent(smr_type='Gaussian', **p),
                    'opt': M.OpticalConductivity(**p)}
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=(3, 4, 2)), mk(C), precision=precision)
    ref = O.run(o, (2, 2, 2), (3, 4, 2), mk(O))
    for q in ('jdos', 'shift', 'inj', 'opt'):
        _close(res[q].data, ref[q].data, tol)


def test_dynamic_argument_errors(golden_dir):
    """qiao / ryoo need the external terms (formula/covariant.py:730-732, 747-749)."""
    s = _random_system(golden_dir)
    with pytest.raises(NotImplementedError):
        wbgpu.run(s, wbgpu.Grid(s, NKdiv=1, NKFFT=2),
                  {'shc': C.SHC(SHC_type='qiao', Efermi=[0.0], omega=[1.0], kwargs_formula={'external_terms': False})})
    with pytest.raises(ValueError):
        C.SHC(SHC_type='other', Efermi=[0.0], omega=[1.0])


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-8), ('mixed', 1e-6)])
def test_static_extra_reference_run(golden_dir, precision, tol):
    """Static SHC (SpinOmega, three spin-current kinds), NLDrude_Fermider2 (fder 2), NLAHC_FermiSea
    against the reference's run() on the random system (static_ref.npz)."""
    s = _random_system(golden_dir)
    ref = np.load(os.path.join(golden_dir, 'static_ref.npz'))
    EF = ref['EF']
    st = C.static
    calcs = {'shc_simple': st.SHC(Efermi=EF, kwargs_formula={'spin_current_type': 'simple'}),
             'shc_simple_int': st.SHC(Efermi=EF, kwargs_formula={'spin_current_type': 'simple',
                                                                 'external_terms': False}),
             'shc_qiao': st.SHC(Efermi=EF, kwargs_formula={'spin_current_type': 'qiao'}),
             'shc_ryoo': st.SHC(Efermi=EF, kwargs_formula={'spin_current_type': 'ryoo'}),
             'nldrude2': st.NLDrude_Fermider2(Efermi=EF), 'nlahc': st.NLAHC_FermiSea(Efermi=EF)}
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=3), calcs, precision=precision)
    for q in calcs:
        _close(res[q].data, ref['random_' + q], tol)
