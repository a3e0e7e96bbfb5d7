"""GPU tests of the in-group product formulas (wbg_berry_product; formula/formula.py:121-151
FormulaProduct with the factor lists of formula/covariant.py:798-858):

* products_ref.npz: the reference's run() on its random system (NK 6 = 2 x 3) for
  BerryDipole_FermiSurf (with and without external terms), NLAHC_FermiSurf, NLDrude_FermiSurf,
  Hall_classic_FermiSurf / FermiSea, GME_spin_FermiSurf / FermiSea, GME_orb_FermiSurf, OmegaOmega and
  AHC_Zeeman_spin / orb;
* the oracle on the triclinic MDRS model (nw = 6, anisotropic FFT grid), with the histogram and with
  the tetrahedron method.

FP64 path within 1e-8 of max|ref| (the reference goldens' rule), mixed path within 1e-6.
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


def _close(got, ref, tol, what=''):
    assert got.shape == ref.shape, what
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err <= tol, (what, err)


def _product_calculators(M, EF, spin=True, **kw):
    cs = {'bcd_fsurf': M.BerryDipole_FermiSurf(Efermi=EF, **kw),
          'bcd_fsurf_int': M.BerryDipole_FermiSurf(Efermi=EF, kwargs_formula={'external_terms': False}, **kw),
          'nlahc_fsurf': M.NLAHC_FermiSurf(Efermi=EF, **kw), 'nldrude_fsurf': M.NLDrude_FermiSurf(Efermi=EF, **kw),
          'hall_fsurf': M.Hall_classic_FermiSurf(Efermi=EF, **kw), 'hall_fsea': M.Hall_classic_FermiSea(Efermi=EF, **kw),
          'omegaomega': M.OmegaOmega(Efermi=EF, **kw)}
    cs['gme_orb_fsurf'] = M.GME_orb_FermiSurf(Efermi=EF, **kw)
    cs['ahc_z_orb'] = M.AHC_Zeeman_orb(Efermi=EF, **kw)
    if spin:
        cs['gme_spin_fsurf'] = M.GME_spin_FermiSurf(Efermi=EF, **kw)
        cs['gme_spin_fsea'] = M.GME_spin_FermiSea(Efermi=EF, **kw)
        cs['ahc_z_spin'] = M.AHC_Zeeman_spin(Efermi=EF, **kw)
    return cs


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-8), ('mixed', 1e-6)])
def test_products_reference_run(golden_dir, precision, tol):
    """Every product calculator against the reference's run() on the random system."""
    s = _random_system(golden_dir)
    ref = np.load(os.path.join(golden_dir, 'products_ref.npz'))
    calcs = _product_calculators(C, ref['EF'])
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=3), calcs, precision=precision)
    for q in calcs:
        _close(res[q].data, ref['random_' + q], tol, q)


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-8), ('mixed', 1e-6)])
def test_products_mdrs_vs_oracle(precision, tol):
    """The product calculators without spin on the triclinic MDRS model (anisotropic FFT grid)
    against the oracle: full O, W, B and C blocks of degenerate groups, the Fermi-sea MassMass group."""
    d = models.config_system(2, small=True)
    s = wsys.System_R.from_dict(d)
    s.do_ws_dist(3)
    o = O.RSystem(s.real_lattice, s.iRvec, s.wannier_centers_cart, s._XX_R)
    EF = np.linspace(-1.0, 1.0, 21)
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=(3, 4, 2)), _product_calculators(C, EF, spin=False),
                    precision=precision)
    ref = O.run(o, (2, 2, 2), (3, 4, 2), _product_calculators(O, EF, spin=False))
    for q in ref:
        _close(res[q].data, ref[q].data, tol, q)


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-8), ('mixed', 1e-6)])
def test_products_tetra_vs_oracle(precision, tol):
    """tetra=True: per-band product values (wbg_product_values) weighted by the tetrahedron
    occupations, Fermi surface and Fermi sea, against the oracle."""
    d = models.config_system(2, small=True)
    s = wsys.System_R.from_dict(d)
    s.do_ws_dist(3)
    o = O.RSystem(s.real_lattice, s.iRvec, s.wannier_centers_cart, s._XX_R)
    EF = np.linspace(-1.0, 1.0, 11)
    mk = lambda M: {'bcd_fsurf': M.BerryDipole_FermiSurf(Efermi=EF, tetra=True),
                    'hall_fsea': M.Hall_classic_FermiSea(Efermi=EF, tetra=True),
                    'nldrude_fsurf': M.NLDrude_FermiSurf(Efermi=EF, tetra=True)}
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=(3, 4, 2)), mk(C), precision=precision)
    ref = O.run(o, (2, 2, 2), (3, 4, 2), mk(O))
    for q in ref:
        _close(res[q].data, ref[q].data, tol, q)
