"""The drop-in boundary, end to end: the reference's own run() (run_grid.py:118-403) with
data_k_class=Data_K_GPU evaluates every block on the GPU through libwbgpu.so, and its results equal
the reference's stored goldens and its own CPU run() on the same systems.

Needs the unmodified reference in baseline/_ref (python baseline/install_reference.py); skipped
without it.  FP64 path: the goldens' 1e-8 acceptance rule, 1e-9 against the CPU run(); mixed path:
1e-6 relative (the precision target of the mixed path).
"""
import os

import numpy as np
import pytest

import refbind_util as RU

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

wb = RU.import_reference()
if wb is None:
    pytest.skip("the reference package is not installed in baseline/_ref", allow_module_level=True)

from wannierberri import calculators as RC  # noqa: E402
from wbgpu import models, system as wsys  # noqa: E402
from wbgpu.refbind import Data_K_GPU  # noqa: E402


def maxrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def random_ref(golden_dir):
    f = np.load(os.path.join(golden_dir, 'random_system.npz'))
    XX = {k[5:]: f[k] for k in f.files if k.startswith('XX_R_')}
    d = dict(real_lattice=f['real_lattice'], iRvec=f['iRvec'], wannier_centers_cart=f['wannier_centers_cart'], XX_R=XX)
    return RU.ref_system(d), np.load(os.path.join(golden_dir, 'random_results.npz'))


@pytest.fixture(scope="module")
def c2small_ref():
    """The small triclinic MDRS model (the structure of the nw=32 benchmark model)."""
    s = wsys.System_R.from_dict(models.config_system(2, small=True))
    s.do_ws_dist(3)
    d = dict(real_lattice=s.real_lattice, iRvec=s.iRvec, wannier_centers_cart=s.wannier_centers_cart,
             XX_R={k: s._XX_R[k] for k in ('Ham', 'AA', 'BB', 'CC')})
    return RU.ref_system(d)


def test_reference_goldens_through_drop_in(random_ref):
    """The reference's golden random-{ahc,Morb,opt_conductivity,dos,cumdos} (settings of
    tests/test_run.py:653-669) reproduced by the reference's run() on Data_K_GPU."""
    system, gold = random_ref
    EF = np.linspace(-2, 2, 5)
    calcs = {'ahc': RC.static.AHC(Efermi=EF), 'Morb': RC.static.Morb(Efermi=EF),
             'dos': RC.static.DOS(Efermi=EF), 'cumdos': RC.static.CumDOS(Efermi=EF),
             'opt_conductivity': RC.dynamic.OpticalConductivity(Efermi=np.array([17.0, 18.0]),
                                                                 omega=np.arange(0.0, 7.1, 1.0), smr_fixed_width=0.20,
                                                                 smr_type="Gaussian")}
    res = RU.ref_run(wb, system, (2, 2, 2), (3, 3, 3), calcs, data_k_class=Data_K_GPU)
    for key in calcs:
        got = res.results[key].data
        exp = gold[key + '_data']
        assert got.shape == exp.shape, key
        assert np.max(np.abs(got - exp)) <= 1e-8 * np.max(np.abs(exp)), (key, maxrel(got, exp))


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-9), ('mixed', 1e-6)])
def test_drop_in_equals_reference_cpu_run(c2small_ref, precision, tol):
    """AHC, Morb, BerryDipole_FermiSea / FermiSurf, Hall_classic_FermiSea, GME_orb_FermiSurf and
    OpticalConductivity of the reference's run() on the MDRS model: Data_K_GPU against the
    reference's own Data_K_R, block by block summed by the driver."""
    system = c2small_ref
    EF = np.linspace(-2, 2, 101)
    mk = lambda: {'ahc': RC.static.AHC(Efermi=EF), 'morb': RC.static.Morb(Efermi=EF),
                  'bcd': RC.static.BerryDipole_FermiSea(Efermi=EF),
                  'bcd_fsurf': RC.static.BerryDipole_FermiSurf(Efermi=EF),
                  'hall_fsea': RC.static.Hall_classic_FermiSea(Efermi=EF),
                  'gme_orb': RC.static.GME_orb_FermiSurf(Efermi=EF),
                  'opt': RC.dynamic.OpticalConductivity(Efermi=np.linspace(-1, 1, 5), omega=np.linspace(0, 3, 20),
                                                        smr_fixed_width=0.1)}
    cpu = RU.ref_run(wb, system, (2, 1, 2), (3, 4, 3), mk())
    gpu = RU.ref_run(wb, system, (2, 1, 2), (3, 4, 3), mk(), data_k_class=Data_K_GPU,
                     parameters_K={'precision': precision})
    for key in ('ahc', 'morb', 'bcd', 'bcd_fsurf', 'hall_fsea', 'gme_orb', 'opt'):
        a, b = gpu.results[key], cpu.results[key]
        assert a.data.shape == b.data.shape, key
        assert maxrel(a.data, b.data) < tol, (key, maxrel(a.data, b.data))
        # the result object is the reference's own, with the formula's symmetry transformations
        assert type(a) is type(b)
        assert a.transformTR.as_dict() == b.transformTR.as_dict(), key
        assert a.transformInv.as_dict() == b.transformInv.as_dict(), key


def test_drop_in_refinement_and_unsupported(c2small_ref):
    """The reference's adaptive refinement (run_grid.py:370-389) re-creates Data_K_GPU for the
    divided K-points; a calculator without a GPU kernel raises instead of running on the CPU."""
    system = c2small_ref
    EF = np.linspace(-2, 2, 41)
    cpu = RU.ref_run(wb, system, (2, 2, 2), (3, 3, 3), {'ahc': RC.static.AHC(Efermi=EF)}, adpt_num_iter=2)
    gpu = RU.ref_run(wb, system, (2, 2, 2), (3, 3, 3), {'ahc': RC.static.AHC(Efermi=EF)}, adpt_num_iter=2,
                     data_k_class=Data_K_GPU)
    assert maxrel(gpu.results['ahc'].data, cpu.results['ahc'].data) < 1e-9
    with pytest.raises(NotImplementedError):
        RU.ref_run(wb, system, (1, 1, 1), (3, 3, 3), {'d': RC.static.NLDrude_FermiSea(Efermi=EF)},
                   data_k_class=Data_K_GPU)
