"""Pin the CPU oracle against the reference's own golden vectors (CPU only).

* tests/reference/integrate_files/random-*_iter-0000.npz with the settings of
  the reference's tests/test_run.py:653-669 (NK=6, NKFFT=3).
* tests/reference/formula/*.npz with the settings of tests/test_formula.py:18-41,171-213.
* reference outputs on seeded synthetic models (tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

from oracle import wb_oracle as O
from wbgpu import models


def load_system(path, prefix=''):
    f = np.load(path)
    XX = {k[len(prefix) + 5:]: f[k] for k in f.files if k.startswith(prefix + 'XX_R_')}
    return O.RSystem(f[prefix + 'real_lattice'], f[prefix + 'iRvec'], f[prefix + 'wannier_centers_cart'], XX)


def maxrel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.fixture(scope="module")
def random_sys(golden_dir):
    return load_system(os.path.join(golden_dir, 'random_system.npz'))


@pytest.fixture(scope="module")
def random_res(golden_dir):
    return np.load(os.path.join(golden_dir, 'random_results.npz'))


@pytest.fixture(scope="module")
def random_run(random_sys, random_res):
    EF = np.linspace(-2, 2, 5)
    calcs = {'ahc': O.AHC(Efermi=EF), 'Morb': O.Morb(Efermi=EF), 'dos': O.DOS(Efermi=EF), 'cumdos': O.CumDOS(Efermi=EF),
             'conductivity_ohmic': O.Ohmic_FermiSea(Efermi=EF), 'conductivity_ohmic_fsurf': O.Ohmic_FermiSurf(Efermi=EF),
             'spin': O.Spin(Efermi=EF)}
    popt = dict(Efermi=np.array([17.0, 18.0]), omega=np.arange(0.0, 7.1, 1.0), smr_fixed_width=0.20,
                smr_type="Gaussian")
    calcs['opt_conductivity'] = O.OpticalConductivity(**popt)
    calcs['opt_SHCqiao'] = O.SHC(SHC_type="qiao", **popt)
    calcs['opt_SHCryoo'] = O.SHC(SHC_type="ryoo", **popt)
    return O.run(random_sys, NKdiv=(2, 2, 2), NKFFT=(3, 3, 3), calculators=calcs)


@pytest.mark.parametrize("quant", ['ahc', 'Morb', 'opt_conductivity', 'dos', 'cumdos', 'conductivity_ohmic',
                                   'conductivity_ohmic_fsurf', 'spin', 'opt_SHCqiao', 'opt_SHCryoo'])
def test_random_golden(random_run, random_res, quant):
    """Same acceptance rule as the reference: abs err < 1e-8 * max|ref| (tests/common_comparers.py:189-196)."""
    ref = random_res[quant + '_data']
    got = random_run[quant].data
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) < 1e-8 * np.max(np.abs(ref))


FORMULAE_LN = ['Dcov', 'DerDcov', 'DEinv_ln']
FORMULAE_NN = ['Omega', 'DerOmega', 'Morb_H']


@pytest.fixture(scope="module")
def fe_datak(golden_dir):
    s = load_system(os.path.join(golden_dir, 'fe_system.npz'))
    return O.DataK(s, NKFFT=(1, 2, 3), dK=(0, 0, 0))


@pytest.mark.parametrize("name", FORMULAE_LN + FORMULAE_NN)
def test_fe_formula_golden(fe_datak, golden_dir, name):
    """tests/test_formula.py:171-220 with its tolerances."""
    data = fe_datak
    ref = np.load(os.path.join(golden_dir, 'fe_formula.npz'))
    cls = {'Dcov': lambda d: d.Dcov, 'DerDcov': O.DerDcov, 'DEinv_ln': O.DEinv_ln,
           'Omega': O.Omega, 'DerOmega': O.DerOmega, 'Morb_H': O.Morb_H}[name]
    NB = data.num_wann
    value = {}
    for ik in range(data.nk):
        groups = data.get_bands_in_range_groups_ik(ik, -10, 30, degen_thresh=1)
        acc = {k: [] for k in ["Xnn", "Xll", "XlnXnl", "XnlXln", "XnnXnn", "XllXll"]}
        for n in groups:
            inn = np.arange(n[0], n[1])
            out = np.concatenate((np.arange(0, n[0]), np.arange(n[1], NB)))
            form = cls(data)
            if name not in FORMULAE_NN:
                Xnl = form.ln(ik, inn, out)
                Xln = form.ln(ik, out, inn)
                acc["XnlXln"].append(np.einsum("nl...,ln...->...", Xnl, Xln))
                acc["XlnXnl"].append(np.einsum("ln...,nl...->...", Xln, Xnl))
            if name not in FORMULAE_LN:
                Xll = form.ll(ik, inn, inn)
                Xnn = form.nn(ik, inn, inn)
                acc["Xll"].append(np.einsum("ll...->...", Xll))
                acc["Xnn"].append(np.einsum("nn...->...", Xnn))
                acc["XllXll"].append(np.einsum("ll...,ll...->...", Xll, Xll))
                acc["XnnXnn"].append(np.einsum("nn...,nn...->...", Xnn, Xnn))
        for k, v in acc.items():
            value[f"{k}_ik={ik}"] = np.array(v)
    rel_tol, atol_zero = (1e-5, 2e-6) if "Der" in name else (1e-6, 1e-10)
    keys = [k for k in ref.files if k.startswith(name + '/')]
    assert keys
    for key in keys:
        val = ref[key]
        out = value[key.split('/', 1)[1]]
        assert out.shape == val.shape
        if val.size == 0:
            continue
        mx = np.max(abs(val))
        if mx < atol_zero:
            assert np.max(abs(out)) < atol_zero
        else:
            assert np.max(abs(val - out)) / mx < rel_tol, key


@pytest.fixture(scope="module")
def synth(golden_dir):
    return np.load(os.path.join(golden_dir, 'synthetic_ref.npz'))


def rsys(d):
    return O.RSystem(d['real_lattice'], d['iRvec'], d['wannier_centers_cart'], d['XX_R'])


def test_synthetic_c1_block(synth):
    """One full-size config-1 block (nw=8, 125 R, 8^3 k at a generic shift): energies and AHC."""
    s = rsys(models.config_system(1))
    data = O.DataK(s, NKFFT=(8, 8, 8), dK=synth['c1_block_dK'])
    assert np.max(np.abs(data.E_K - synth['c1_block_E'])) < 1e-10
    ahc = O.AHC(Efermi=np.linspace(-2, 2, 501))(data).data
    assert maxrel(ahc, synth['c1_block_ahc']) < 1e-10


def test_synthetic_c1_run(synth):
    s = rsys(models.config_system(1))
    r = O.run(s, (2, 2, 2), (4, 4, 4), {'ahc': O.AHC(Efermi=np.linspace(-2, 2, 41))})
    assert maxrel(r['ahc'].data, synth['c1_run_ahc']) < 1e-10


def test_synthetic_c2_mdrs_and_run(synth):
    s = rsys(models.config_system(2, small=True))
    s2 = O.do_ws_dist(s, mp_grid=(3, 3, 3))
    # same replica set and matrices (order-independent comparison)
    ref_R = synth['c2_mdrs_iRvec']
    idx = {tuple(R): i for i, R in enumerate(s2.iRvec)}
    assert len(idx) == len(ref_R)
    perm = np.array([idx[tuple(R)] for R in ref_R])
    for k in ['Ham', 'AA', 'BB', 'CC']:
        assert np.max(np.abs(s2.XX_R[k][perm] - synth['c2_mdrs_' + k])) < 1e-12
    EF = np.linspace(-2, 2, 41)
    r = O.run(s2, (2, 2, 2), (4, 4, 4), {'ahc': O.AHC(Efermi=EF), 'morb': O.Morb(Efermi=EF),
                                         'bcd': O.BerryDipole_FermiSea(Efermi=EF)})
    for k in ['ahc', 'morb', 'bcd']:
        assert maxrel(r[k].data, synth['c2_run_' + k]) < 1e-9, k


def test_synthetic_c3_run(synth):
    s = rsys(models.config_system(3, small=True))
    EF3 = np.linspace(-1, 1, 11)
    om = np.linspace(0, 4, 40)
    r = O.run(s, (2, 2, 2), (4, 4, 4), {'opt': O.OpticalConductivity(Efermi=EF3, omega=om, smr_fixed_width=0.05),
                                        'ahc': O.AHC(Efermi=EF3)})
    assert maxrel(r['opt'].data, synth['c3_run_opt']) < 1e-10
    assert maxrel(r['ahc'].data, synth['c3_run_ahc']) < 1e-9


EVK_QS = ['energy', 'band_gradients', 'berry_curvature', 'berry_curvature_internal_terms',
          'berry_curvature_external_terms']


def test_oracle_evaluate_k_golden(golden_dir):
    """The oracle's evaluate_k against the reference's own evaluate_k (random system at three
    k-points, Fe at one k-point, bands 4-5); acceptance of tests/test_evaluate_k.py: rel 1e-8."""
    import os
    g = np.load(os.path.join(golden_dir, 'evaluate_k_ref.npz'))
    f = np.load(os.path.join(golden_dir, 'random_system.npz'))
    rs = O.RSystem(f['real_lattice'], f['iRvec'], f['wannier_centers_cart'],
                   {k[5:]: f[k] for k in f.files if k.startswith('XX_R_')})
    for i, kp in enumerate(g['random_k']):
        got = O.evaluate_k(rs, kp, EVK_QS)
        for q in EVK_QS:
            ref = g[f'random_{i}_{q}']
            assert np.allclose(got[q], ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max()), (i, q)
    f = np.load(os.path.join(golden_dir, 'fe_system.npz'))
    fe = O.RSystem(f['real_lattice'], f['iRvec'], f['wannier_centers_cart'],
                   {k[5:]: f[k] for k in f.files if k.startswith('XX_R_')})
    got = O.evaluate_k(fe, g['fe_k'], EVK_QS, iband=[4, 5])
    for q in EVK_QS:
        ref = g[f'fe_{q}']
        assert np.allclose(got[q], ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max()), q


def tetra_oracle_calculators(EF, names):
    """tetra=True static calculators of the oracle, the same set as tests/golden/make_golden.py."""
    cs = {'ahc': O.AHC, 'morb': O.Morb, 'bcd': O.BerryDipole_FermiSea, 'dos': O.DOS, 'cumdos': O.CumDOS,
          'conductivity_ohmic': O.Ohmic_FermiSea, 'conductivity_ohmic_fsurf': O.Ohmic_FermiSurf}
    return {k: cs[k](Efermi=EF, tetra=True) for k in names}


TETRA_RANDOM = ['ahc', 'morb', 'bcd', 'dos', 'cumdos', 'conductivity_ohmic', 'conductivity_ohmic_fsurf']


def test_tetra_random_golden(random_sys, golden_dir):
    """Tetrahedron method (grid/tetrahedron.py TetraWeightsParal, corner energies of
    data_K/data_K_R.py:121-141) against the reference's run on its random system."""
    g = np.load(os.path.join(golden_dir, 'tetra_ref.npz'))
    r = O.run(random_sys, NKdiv=(2, 2, 2), NKFFT=(3, 3, 3), calculators=tetra_oracle_calculators(g['EF'], TETRA_RANDOM))
    for k in TETRA_RANDOM:
        ref = g['random_' + k]
        assert r[k].data.shape == ref.shape, k
        assert np.max(np.abs(r[k].data - ref)) < 1e-8 * np.max(np.abs(ref)), k


def test_tetra_c2_anisotropic_golden(golden_dir):
    """Triclinic MDRS model over NKdiv (2,1,3) x NKFFT (3,4,2): the corner k-points of every
    block cross the block borders in all three directions."""
    g = np.load(os.path.join(golden_dir, 'tetra_ref.npz'))
    s2 = O.do_ws_dist(rsys(models.config_system(2, small=True)), mp_grid=(3, 3, 3))
    names = ['ahc', 'dos', 'conductivity_ohmic']
    r = O.run(s2, (2, 1, 3), (3, 4, 2), tetra_oracle_calculators(g['EF2'], names))
    for k in names:
        assert maxrel(r[k].data, g['c2_' + k]) < 1e-9, k


def test_refine_random_golden(random_sys, golden_dir):
    """Adaptive refinement (run_grid.py:290-403 without symmetry) against the reference's run on
    its random system: 3 iterations, the largest K-point per ResultDict.max entry divided into 2^3."""
    g = np.load(os.path.join(golden_dir, 'refine_ref.npz'))
    EF = g['EF']
    calcs = {'ahc': O.AHC(Efermi=EF), 'dos': O.DOS(Efermi=EF), 'cumdos': O.CumDOS(Efermi=EF)}
    r, (K, dK, fac) = O.run_adaptive(random_sys, (2, 2, 2), (3, 3, 3), calcs, adpt_num_iter=3, adpt_mesh=2)
    assert abs(fac.sum() - 1.0) < 1e-12 and len(K) > 8
    for k in calcs:
        ref = g['random_' + k]
        assert np.max(np.abs(r[k].data - ref)) < 1e-8 * np.max(np.abs(ref)), k


def test_refine_c2_anisotropic_golden(golden_dir):
    """Triclinic MDRS model, adpt_fac 2, adpt_mesh (2, 1, 3) over NKdiv 2 x NKFFT (3, 4, 2)."""
    g = np.load(os.path.join(golden_dir, 'refine_ref.npz'))
    s2 = O.do_ws_dist(rsys(models.config_system(2, small=True)), mp_grid=(3, 3, 3))
    EF = g['EF2']
    calcs = {'ahc': O.AHC(Efermi=EF), 'bcd': O.BerryDipole_FermiSea(Efermi=EF)}
    r, _ = O.run_adaptive(s2, (2, 2, 2), (3, 4, 2), calcs, adpt_num_iter=2, adpt_mesh=(2, 1, 3), adpt_fac=2)
    for k in calcs:
        assert maxrel(r[k].data, g['c2_' + k]) < 1e-9, k


def test_refine_tetra_golden(random_sys, golden_dir):
    """Tetrahedron method on refined K-points: each K-point's corners follow its own cell."""
    g = np.load(os.path.join(golden_dir, 'refine_ref.npz'))
    EF = g['EF']
    calcs = {'ahc': O.AHC(Efermi=EF, tetra=True), 'dos': O.DOS(Efermi=EF, tetra=True)}
    r, _ = O.run_adaptive(random_sys, (2, 2, 2), (3, 3, 3), calcs, adpt_num_iter=2, adpt_mesh=2)
    for k in calcs:
        ref = g['tetra_random_' + k]
        assert np.max(np.abs(r[k].data - ref)) < 1e-8 * np.max(np.abs(ref)), k


def dynamic_calculators(EF, om):
    """The calculators of dynamic_ref.npz (tests/golden/make_golden.py, section 7)."""
    pL = dict(Efermi=EF, omega=om, smr_fixed_width=0.3)
    pG = dict(Efermi=EF, omega=om, smr_fixed_width=0.2, smr_type='Gaussian', kBT=0.05)
    return {'jdos_L': O.JDOS(**pL), 'jdos_G': O.JDOS(**pG),
            'shc_simple_L': O.SHC(SHC_type='simple', **pL),
            'shc_simple_int_G': O.SHC(SHC_type='simple', kwargs_formula={'external_terms': False}, **pG),
            'shc_qiao_L': O.SHC(SHC_type='qiao', **pL), 'shc_ryoo_G': O.SHC(SHC_type='ryoo', **pG),
            'shc_ryoo_abc_L': O.SHC(SHC_type='ryoo', shc_abc=(1, 2, 3), **pL),
            'shift_G': O.ShiftCurrent(sc_eta=0.1, **pG),
            'shift_int_L': O.ShiftCurrent(sc_eta=0.1, kwargs_formula={'external_terms': False}, **pL),
            'injection_G': O.InjectionCurrent(**pG), 'injection_L': O.InjectionCurrent(**pL),
            'spin': O.Spin(Efermi=np.linspace(-3, 3, 11))}


@pytest.fixture(scope="module")
def dynamic_ref(golden_dir):
    return np.load(os.path.join(golden_dir, 'dynamic_ref.npz'))


@pytest.fixture(scope="module")
def dynamic_run(random_sys, dynamic_ref):
    return O.run(random_sys, (2, 2, 2), (3, 3, 3), dynamic_calculators(dynamic_ref['EF'], dynamic_ref['omega']))


@pytest.mark.parametrize("quant", ['jdos_L', 'jdos_G', 'shc_simple_L', 'shc_simple_int_G', 'shc_qiao_L', 'shc_ryoo_G',
                                   'shc_ryoo_abc_L', 'shift_G', 'shift_int_L', 'injection_G', 'injection_L', 'spin'])
def test_dynamic_golden(dynamic_run, dynamic_ref, quant):
    """JDOS, SHC, shift and injection currents, Spin: the reference's run() on the random system."""
    ref = dynamic_ref['random_' + quant]
    got = dynamic_run[quant].data
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) < 1e-8 * np.max(np.abs(ref))


def static_calculators(EF):
    """The calculators of static_ref.npz (tests/golden/make_golden.py, section 8)."""
    return {'shc_simple': O.SHC_static(Efermi=EF, kwargs_formula={'spin_current_type': 'simple'}),
            'shc_simple_int': O.SHC_static(Efermi=EF, kwargs_formula={'spin_current_type': 'simple',
                                                                      'external_terms': False}),
            'shc_qiao': O.SHC_static(Efermi=EF, kwargs_formula={'spin_current_type': 'qiao'}),
            'shc_ryoo': O.SHC_static(Efermi=EF, kwargs_formula={'spin_current_type': 'ryoo'}),
            'nldrude2': O.NLDrude_Fermider2(Efermi=EF), 'nlahc': O.NLAHC_FermiSea(Efermi=EF)}


@pytest.fixture(scope="module")
def static_ref(golden_dir):
    return np.load(os.path.join(golden_dir, 'static_ref.npz'))


@pytest.fixture(scope="module")
def static_run(random_sys, static_ref):
    return O.run(random_sys, (2, 2, 2), (3, 3, 3), static_calculators(static_ref['EF']))


@pytest.mark.parametrize("quant", ['shc_simple', 'shc_simple_int', 'shc_qiao', 'shc_ryoo', 'nldrude2', 'nlahc'])
def test_static_extra_golden(static_run, static_ref, quant):
    """Static SHC (SpinOmega), NLDrude_Fermider2 (fder 2), NLAHC_FermiSea: the reference's run()."""
    ref = static_ref['random_' + quant]
    got = static_run[quant].data
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) < 1e-8 * np.max(np.abs(ref))


def product_calculators(EF):
    """The calculators of products_ref.npz (tests/golden/make_golden.py, section 9)."""
    return {'bcd_fsurf': O.BerryDipole_FermiSurf(Efermi=EF),
            'bcd_fsurf_int': O.BerryDipole_FermiSurf(Efermi=EF, kwargs_formula={'external_terms': False}),
            'nlahc_fsurf': O.NLAHC_FermiSurf(Efermi=EF), 'nldrude_fsurf': O.NLDrude_FermiSurf(Efermi=EF),
            'hall_fsurf': O.Hall_classic_FermiSurf(Efermi=EF), 'hall_fsea': O.Hall_classic_FermiSea(Efermi=EF),
            'nldrude_fsea': O.NLDrude_FermiSea(Efermi=EF), 'gme_spin_fsurf': O.GME_spin_FermiSurf(Efermi=EF),
            'gme_spin_fsea': O.GME_spin_FermiSea(Efermi=EF), 'gme_orb_fsurf': O.GME_orb_FermiSurf(Efermi=EF),
            'omegaomega': O.OmegaOmega(Efermi=EF), 'ahc_z_spin': O.AHC_Zeeman_spin(Efermi=EF),
            'ahc_z_orb': O.AHC_Zeeman_orb(Efermi=EF), 'gme_orb_fsea': O.GME_orb_FermiSea(Efermi=EF),
            'gme_orb_fsea_int': O.GME_orb_FermiSea(Efermi=EF, kwargs_formula={'external_terms': False})}


@pytest.fixture(scope="module")
def products_ref(golden_dir):
    return np.load(os.path.join(golden_dir, 'products_ref.npz'))


@pytest.fixture(scope="module")
def products_run(random_sys, products_ref):
    return O.run(random_sys, (2, 2, 2), (3, 3, 3), product_calculators(products_ref['EF']))


@pytest.mark.parametrize("quant", ['bcd_fsurf', 'bcd_fsurf_int', 'nlahc_fsurf', 'nldrude_fsurf', 'hall_fsurf',
                                   'hall_fsea', 'nldrude_fsea', 'gme_spin_fsurf', 'gme_spin_fsea', 'gme_orb_fsurf',
                                   'omegaomega', 'ahc_z_spin', 'ahc_z_orb', 'gme_orb_fsea', 'gme_orb_fsea_int'])
def test_product_formulas_golden(products_run, products_ref, quant):
    """In-group matrix products (VelOmega, MassVel, VelMassVel, MassMass), the classical Hall
    antisymmetrisations and the third derivative of E (Der3E): the reference's run() on the
    random system."""
    ref = products_ref['random_' + quant]
    got = products_run[quant].data
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) < 1e-8 * np.max(np.abs(ref))
