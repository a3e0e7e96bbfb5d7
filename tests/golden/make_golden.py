"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run in a container where the reference (wannier-berri) source tree is mounted:

    python tests/golden/make_golden.py /root/reference

It imports the reference with two tiny shims (``termcolor.cprint`` -> print,
``numba.njit`` -> identity; neither is on the hot path) and with
PYTHONDONTWRITEBYTECODE so nothing is written into the reference tree.

Fixtures written (all small, complex128/float64):

* ``random_system.npz`` + ``random_results.npz`` -- the reference's own test
  system ``tests/data/random`` (nw=6, nR=20) and its stored golden results
  ``tests/reference/integrate_files/random-{ahc,Morb,opt_conductivity,dos,cumdos,
  conductivity_ohmic,conductivity_ohmic_fsurf,spin,opt_SHCqiao,opt_SHCryoo}_iter-0000.npz``
  (settings of ``tests/test_run.py:653-669``: NK=6, NKFFT=3, E_F=linspace(-2,2,5)).
* ``fe_system.npz`` + ``fe_formula.npz`` -- ``tests/reference/systems/system_Fe_sym_W90_OSD``
  (Ham, AA, BB, CC only) and the stored formula traces
  ``tests/reference/formula/{Omega,DerOmega,Morb_H,Dcov,DerDcov,DEinv_ln}.npz``
  (settings of ``tests/test_formula.py:18-41,171-213``).
* ``evaluate_k_ref.npz`` -- the reference's ``evaluate_k`` (energy, band_gradients,
  berry_curvature and its internal / external parts) on the random system at three
  k-points and on the Fe system at k = (0.1, 0.2, 0.3), bands 4 and 5.
* ``synthetic_ref.npz`` -- outputs of the reference's ``wannierberri.run`` /
  ``Data_K_R`` on small seeded models with the structure of the benchmark
  configurations (cubic nw=8 / triclinic nw=6 with MDRS / spinor nw=8), made by
  ``wbgpu.models``: per-block E_K, and AHC / Morb / BerryDipole_FermiSea /
  OpticalConductivity results.
* ``tetra_ref.npz`` -- the tetrahedron method (``tetra=True``: AHC, Morb,
  BerryDipole_FermiSea, DOS, CumDOS, Ohmic_FermiSea / FermiSurf) of the reference's
  ``run`` on the random system (NKdiv 2, NKFFT 3, 21 Fermi levels) and AHC / DOS /
  Ohmic_FermiSea on the triclinic MDRS model over an anisotropic grid (NKdiv (2,1,3),
  NKFFT (3,4,2)).  ``python make_golden.py <reference root> tetra`` writes only this file.
* ``refine_ref.npz`` -- adaptive refinement (``adpt_num_iter``) of the reference's ``run``
  without symmetry: the random system (3 iterations, AHC / DOS / CumDOS) and the triclinic
  MDRS model (2 iterations, adpt_fac 2, adpt_mesh (2,1,3), AHC / BerryDipole_FermiSea), and
  AHC / DOS with tetra=True on the random system (2 iterations).
  ``python make_golden.py <reference root> refine`` writes only this file.
* ``dynamic_ref.npz`` -- JDOS, SHC (simple / qiao / ryoo, one shc_abc component),
  ShiftCurrent, InjectionCurrent and the static Spin of the reference's ``run`` on the random
  system (NKdiv 2, NKFFT 3), Lorentzian and Gaussian smearing.
  ``python make_golden.py <reference root> dynamic`` writes only this file; ``random`` rewrites
  only the random-system files (its spin matrices and the stored spin / SHC results included).
* ``static_ref.npz`` -- the static SHC (SpinOmega; simple, simple without external terms, qiao,
  ryoo), NLDrude_Fermider2 and NLAHC_FermiSea of the reference's ``run`` on the random system.
  ``python make_golden.py <reference root> static`` writes only this file.
* ``products_ref.npz`` -- the product-formula calculators of calculators/static.py
  (BerryDipole_FermiSurf with and without external terms, NLAHC_FermiSurf, NLDrude_FermiSurf,
  Hall_classic_FermiSurf, Hall_classic_FermiSea), NLDrude_FermiSea (the covariant third
  derivative of the energy), the gyrotropic GME_spin_FermiSurf / FermiSea and GME_orb_FermiSurf /
  FermiSea (the latter with and without external terms),
  OmegaOmega and the Zeeman AHC corrections AHC_Zeeman_spin / orb of the reference's ``run`` on
  the random system.
  ``python make_golden.py <reference root> products`` writes only this file.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def setup_reference(ref_root):
    os.environ['PYTHONDONTWRITEBYTECODE'] = '1'
    sys.dont_write_bytecode = True
    shim = tempfile.mkdtemp(prefix='wbshim_')
    os.makedirs(os.path.join(shim, 'termcolor'))
    os.makedirs(os.path.join(shim, 'numba'))
    with open(os.path.join(shim, 'termcolor', '__init__.py'), 'w') as f:
        f.write("def cprint(*a, **k):\n    print(a[0] if a else '')\n"
                "def colored(s, *a, **k):\n    return s\n")
    with open(os.path.join(shim, 'numba', '__init__.py'), 'w') as f:
        f.write("def njit(*a, **k):\n    if len(a) == 1 and callable(a[0]) and not k:\n        return a[0]\n"
                "    return lambda f: f\njit = njit\n")
    sys.path.insert(0, shim)
    sys.path.insert(0, ref_root)
    sys.path.insert(0, os.path.join(REPO, 'wannier-berri_gb300'))
    import wannierberri  # noqa: F401
    return wannierberri


def ref_system_from_arrays(wb, d):
    from wannierberri.system.system_R import System_R
    from wannierberri.fourier.rvectors import Rvectors
    s = System_R(silent=True)
    s.set_real_lattice(real_lattice=d['real_lattice'])
    s.num_wann = d['XX_R']['Ham'].shape[1]
    s.set_wannier_centers(wannier_centers_cart=d['wannier_centers_cart'])
    s.rvec = Rvectors(lattice=s.real_lattice, iRvec=d['iRvec'], shifts_left_red=s.wannier_centers_red)
    for k, v in d['XX_R'].items():
        s.set_R_mat(k, v.copy())
    s.do_at_end_of_init()
    return s


def pack_system(prefix, s, keys):
    out = {prefix + 'real_lattice': s.real_lattice, prefix + 'iRvec': s.rvec.iRvec,
           prefix + 'wannier_centers_cart': s.wannier_centers_cart}
    for k in keys:
        out[prefix + 'XX_R_' + k] = s.get_R_mat(k)
    return out


def run_ref(wb, system, NKdiv, NKFFT, calculators):
    from wannierberri.grid import Grid
    tmp = tempfile.mkdtemp(prefix='wbrun_')
    grid = Grid(system=system, NKdiv=NKdiv, NKFFT=NKFFT, use_symmetry=False)
    res = wb.run(system, grid=grid, calculators=calculators, parallel=False, use_irred_kpt=False,
                 symmetrize=False, fout_name=os.path.join(tmp, 'r'), file_Klist_path=os.path.join(tmp, 'k'),
                 print_progress_step_time=1e9)
    return {k: res.results[k].data for k in calculators}


RANDOM_KEYS = ['Ham', 'AA', 'BB', 'CC', 'SS', 'SA', 'SHA', 'SR', 'SH', 'SHR']
RANDOM_RESULTS = ['ahc', 'Morb', 'opt_conductivity', 'dos', 'cumdos', 'conductivity_ohmic',
                  'conductivity_ohmic_fsurf', 'spin', 'opt_SHCqiao', 'opt_SHCryoo']


def random_fixtures(ref_root):
    """---- 1. the reference's random test system (with its spin matrices) and its stored
    results of tests/test_run.py:653-669."""
    from wannierberri.system.system_R import System_R
    rs = System_R.from_npz(path=os.path.join(ref_root, 'tests', 'data', 'random'), legacy=True)
    np.savez_compressed(os.path.join(HERE, 'random_system.npz'), **pack_system('', rs, RANDOM_KEYS))
    res = {}
    for q in RANDOM_RESULTS:
        f = np.load(os.path.join(ref_root, 'tests', 'reference', 'integrate_files', f'random-{q}_iter-0000.npz'),
                    allow_pickle=True)
        res[q + '_data'] = f['data']
        res[q + '_E0'] = f['Energies_0']
        if 'Energies_1' in f:
            res[q + '_E1'] = f['Energies_1']
    np.savez_compressed(os.path.join(HERE, 'random_results.npz'), **res)
    return rs


def dynamic_fixtures(wb, rs):
    """---- 7. dynamic calculators (calculators/dynamic.py) and the static Spin of the
    reference's run on the random system (NKdiv 2 x NKFFT 3): JDOS, SHC of the three
    spin-current kinds (and one shc_abc component), ShiftCurrent and InjectionCurrent, with
    Lorentzian and Gaussian smearing, at zero and finite temperature."""
    from wannierberri import calculators as calc
    dyn = calc.dynamic
    out = {}
    EF = np.array([-1.0, 0.0, 1.0, 2.0])
    om = np.linspace(0.0, 6.0, 13)
    out['EF'], out['omega'] = EF, om
    pL = dict(Efermi=EF, omega=om, smr_fixed_width=0.3)
    pG = dict(Efermi=EF, omega=om, smr_fixed_width=0.2, smr_type='Gaussian', kBT=0.05)
    cs = {'jdos_L': dyn.JDOS(**pL), 'jdos_G': dyn.JDOS(**pG),
          'shc_simple_L': dyn.SHC(SHC_type='simple', **pL),
          'shc_simple_int_G': dyn.SHC(SHC_type='simple', kwargs_formula={'external_terms': False}, **pG),
          'shc_qiao_L': dyn.SHC(SHC_type='qiao', **pL), 'shc_ryoo_G': dyn.SHC(SHC_type='ryoo', **pG),
          'shc_ryoo_abc_L': dyn.SHC(SHC_type='ryoo', shc_abc=(1, 2, 3), **pL),
          'shift_G': dyn.ShiftCurrent(sc_eta=0.1, **pG), 'shift_int_L': dyn.ShiftCurrent(
              sc_eta=0.1, kwargs_formula={'external_terms': False}, **pL),
          'injection_G': dyn.InjectionCurrent(**pG), 'injection_L': dyn.InjectionCurrent(**pL),
          'spin': calc.static.Spin(Efermi=np.linspace(-3, 3, 11))}
    for k, v in run_ref(wb, rs, 2, 3, cs).items():
        out['random_' + k] = v
    np.savez_compressed(os.path.join(HERE, 'dynamic_ref.npz'), **out)


def static_fixtures(wb, rs):
    """---- 8. more static calculators (calculators/static.py) of the reference's run on the
    random system (NKdiv 2 x NKFFT 3): the static SHC (SpinOmega) of the three spin-current kinds,
    NLDrude_Fermider2 (fder 2) and NLAHC_FermiSea."""
    from wannierberri import calculators as calc
    st = calc.static
    EF = np.linspace(-2, 2, 21)
    out = {'EF': EF}
    cs = {'shc_simple': st.SHC(Efermi=EF, kwargs_formula={'spin_current_type': 'simple'}),
          'shc_simple_int': st.SHC(Efermi=EF, kwargs_formula={'spin_current_type': 'simple', 'external_terms': False}),
          'shc_qiao': st.SHC(Efermi=EF, kwargs_formula={'spin_current_type': 'qiao'}),
          'shc_ryoo': st.SHC(Efermi=EF, kwargs_formula={'spin_current_type': 'ryoo'}),
          'nldrude2': st.NLDrude_Fermider2(Efermi=EF), 'nlahc': st.NLAHC_FermiSea(Efermi=EF)}
    for k, v in run_ref(wb, rs, 2, 3, cs).items():
        out['random_' + k] = v
    np.savez_compressed(os.path.join(HERE, 'static_ref.npz'), **out)


def products_fixtures(wb, rs):
    """---- 9. product formulas (formula/formula.py FormulaProduct: in-group matrix products) of the
    reference's run on the random system (NKdiv 2 x NKFFT 3, 21 Fermi levels)."""
    from wannierberri import calculators as calc
    st = calc.static
    EF = np.linspace(-2, 2, 21)
    out = {'EF': EF}
    cs = {'bcd_fsurf': st.BerryDipole_FermiSurf(Efermi=EF),
          'bcd_fsurf_int': st.BerryDipole_FermiSurf(Efermi=EF, kwargs_formula={'external_terms': False}),
          'nlahc_fsurf': st.NLAHC_FermiSurf(Efermi=EF), 'nldrude_fsurf': st.NLDrude_FermiSurf(Efermi=EF),
          'hall_fsurf': st.Hall_classic_FermiSurf(Efermi=EF), 'hall_fsea': st.Hall_classic_FermiSea(Efermi=EF),
          'nldrude_fsea': st.NLDrude_FermiSea(Efermi=EF), 'gme_spin_fsurf': st.GME_spin_FermiSurf(Efermi=EF),
          'gme_spin_fsea': st.GME_spin_FermiSea(Efermi=EF), 'gme_orb_fsurf': st.GME_orb_FermiSurf(Efermi=EF),
          'omegaomega': st.OmegaOmega(Efermi=EF), 'ahc_z_spin': st.AHC_Zeeman_spin(Efermi=EF),
          'ahc_z_orb': st.AHC_Zeeman_orb(Efermi=EF), 'gme_orb_fsea': st.GME_orb_FermiSea(Efermi=EF),
          'gme_orb_fsea_int': st.GME_orb_FermiSea(Efermi=EF, kwargs_formula={'external_terms': False})}
    for k, v in run_ref(wb, rs, 2, 3, cs).items():
        out['random_' + k] = v
    np.savez_compressed(os.path.join(HERE, 'products_ref.npz'), **out)


def main(ref_root):
    wb = setup_reference(ref_root)
    from wannierberri.system.system_R import System_R
    from wannierberri import calculators as calc
    from wbgpu import models

    # ---- 1. the reference's own random system and stored results
    rs = random_fixtures(ref_root)
    # ---- 2. Fe formula system and stored formula traces
    fe = System_R.from_npz(os.path.join(ref_root, 'tests', 'reference', 'systems', 'system_Fe_sym_W90_OSD'),
                           matrices=['Ham', 'AA', 'BB', 'CC'])
    np.savez_compressed(os.path.join(HERE, 'fe_system.npz'), **pack_system('', fe, ['Ham', 'AA', 'BB', 'CC']))
    fres = {}
    for name in ['Omega', 'DerOmega', 'Morb_H', 'Dcov', 'DerDcov', 'DEinv_ln']:
        f = np.load(os.path.join(ref_root, 'tests', 'reference', 'formula', name + '.npz'))
        for k in f.files:
            fres[name + '/' + k] = f[k]
    np.savez_compressed(os.path.join(HERE, 'fe_formula.npz'), **fres)

    # ---- 3. reference outputs on seeded synthetic models
    out = {}
    EF = np.linspace(-2, 2, 41)
    # config-1 structure at full nw=8, R in [-2,2]^3: one 8^3 block at a generic shift + 2^3 blocks of 4^3
    d1 = models.config_system(1)
    s1 = ref_system_from_arrays(wb, d1)
    from wannierberri.data_K.data_K_R import Data_K_R
    from wannierberri.grid import Grid
    g = Grid(system=s1, NKdiv=1, NKFFT=8, use_symmetry=False)
    dK = np.array([0.3, 0.1, 0.7]) / 8
    dk = Data_K_R(s1, dK=dK, grid=g)
    out['c1_block_dK'] = dK
    out['c1_block_E'] = dk.E_K
    ahc = calc.static.AHC(Efermi=np.linspace(-2, 2, 501))
    out['c1_block_ahc'] = ahc(dk).data
    r = run_ref(wb, s1, 2, 4, {'ahc': calc.static.AHC(Efermi=EF)})
    out['c1_run_ahc'] = r['ahc']
    # config-2 structure (triclinic, random centres, BB/CC, MDRS) at small size
    d2 = models.config_system(2, small=True)
    s2 = ref_system_from_arrays(wb, d2)
    s2.do_ws_dist(mp_grid=3)
    out['c2_mdrs_iRvec'] = s2.rvec.iRvec
    for k in ['Ham', 'AA', 'BB', 'CC']:
        out['c2_mdrs_' + k] = s2.get_R_mat(k)
    r = run_ref(wb, s2, 2, 4, {'ahc': calc.static.AHC(Efermi=EF),
                               'morb': calc.static.Morb(Efermi=EF),
                               'bcd': calc.static.BerryDipole_FermiSea(Efermi=EF)})
    for k, v in r.items():
        out['c2_run_' + k] = v
    # config-3 structure (spin-interlaced + SOC) at small size: optical conductivity + AHC
    d3 = models.config_system(3, small=True)
    s3 = ref_system_from_arrays(wb, d3)
    EF3 = np.linspace(-1, 1, 11)
    om = np.linspace(0, 4, 40)
    r = run_ref(wb, s3, 2, 4, {'opt': calc.dynamic.OpticalConductivity(Efermi=EF3, omega=om, smr_fixed_width=0.05),
                               'ahc': calc.static.AHC(Efermi=EF3)})
    for k, v in r.items():
        out['c3_run_' + k] = v
    np.savez_compressed(os.path.join(HERE, 'synthetic_ref.npz'), **out)

    # ---- 4. evaluate_k (evaluate_k.py:33-131) on the random and Fe systems
    ev = {}
    qs = ['energy', 'band_gradients', 'berry_curvature', 'berry_curvature_internal_terms',
          'berry_curvature_external_terms']
    kpts = np.array([[0.1, 0.2, 0.3], [0.0, 0.0, 0.0], [0.45, -0.31, 0.12]])
    ev['random_k'] = kpts
    for i, kp in enumerate(kpts):
        r = wb.evaluate_k(rs, k=kp, quantities=qs, return_single_as_dict=True)
        for q in qs:
            ev[f'random_{i}_{q}'] = r[q]
    fek = np.array([0.1, 0.2, 0.3])
    ev['fe_k'] = fek
    r = wb.evaluate_k(fe, k=fek, quantities=qs, iband=[4, 5], return_single_as_dict=True)
    for q in qs:
        ev[f'fe_{q}'] = r[q]
    np.savez_compressed(os.path.join(HERE, 'evaluate_k_ref.npz'), **ev)
    tetra_fixtures(wb, rs)
    refine_fixtures(wb, rs)
    dynamic_fixtures(wb, rs)
    static_fixtures(wb, rs)
    products_fixtures(wb, rs)
    print("wrote fixtures to", HERE)


def tetra_calculators(calc, EF):
    """Static calculators with tetra=True (calculators/static.py:80-125)."""
    return {'ahc': calc.static.AHC(Efermi=EF, tetra=True),
            'morb': calc.static.Morb(Efermi=EF, tetra=True),
            'bcd': calc.static.BerryDipole_FermiSea(Efermi=EF, tetra=True),
            'dos': calc.static.DOS(Efermi=EF, tetra=True),
            'cumdos': calc.static.CumDOS(Efermi=EF, tetra=True),
            'conductivity_ohmic': calc.static.Ohmic_FermiSea(Efermi=EF, tetra=True),
            'conductivity_ohmic_fsurf': calc.static.Ohmic_FermiSurf(Efermi=EF, tetra=True)}


def tetra_fixtures(wb, rs):
    """---- 5. the tetrahedron method (grid/tetrahedron.py, TetraWeightsParal) on the random
    system (the reference's test grid NK=6 = 2 x 3) and on the config-2 structure with MDRS."""
    from wannierberri import calculators as calc
    from wbgpu import models
    out = {}
    EF = np.linspace(-2, 2, 21)
    out['EF'] = EF
    for k, v in run_ref(wb, rs, 2, 3, tetra_calculators(calc, EF)).items():
        out['random_' + k] = v
    s2 = ref_system_from_arrays(wb, models.config_system(2, small=True))
    s2.do_ws_dist(mp_grid=3)
    EF2 = np.linspace(-1.5, 1.5, 31)
    out['EF2'] = EF2
    cs = tetra_calculators(calc, EF2)
    for k, v in run_ref(wb, s2, [2, 1, 3], [3, 4, 2], {q: cs[q] for q in ('ahc', 'dos', 'conductivity_ohmic')}).items():
        out['c2_' + k] = v
    np.savez_compressed(os.path.join(HERE, 'tetra_ref.npz'), **out)


def run_ref_adaptive(wb, system, NKdiv, NKFFT, calculators, **adpt):
    from wannierberri.grid import Grid
    tmp = tempfile.mkdtemp(prefix='wbrun_')
    grid = Grid(system=system, NKdiv=NKdiv, NKFFT=NKFFT, use_symmetry=False)
    res = wb.run(system, grid=grid, calculators=calculators, parallel=False, use_irred_kpt=False,
                 symmetrize=False, fout_name=os.path.join(tmp, 'r'), file_Klist_path=os.path.join(tmp, 'k'),
                 print_progress_step_time=1e9, **adpt)
    return {k: res.results[k].data for k in calculators}


def refine_fixtures(wb, rs):
    """---- 6. adaptive refinement (run_grid.py:290-403, grid/Kpoint.py:145-175) without
    symmetry: the random system over NKdiv 2 x NKFFT 3 with 3 refinement iterations (AHC, DOS,
    CumDOS; the K-points of largest max(result) x factor divided into 2^3), and the triclinic
    MDRS model with adpt_fac 2 and an anisotropic adpt_mesh (2, 1, 3)."""
    from wannierberri import calculators as calc
    from wbgpu import models
    out = {}
    EF = np.linspace(-2, 2, 21)
    out['EF'] = EF
    cs = {'ahc': calc.static.AHC(Efermi=EF), 'dos': calc.static.DOS(Efermi=EF),
          'cumdos': calc.static.CumDOS(Efermi=EF)}
    for k, v in run_ref_adaptive(wb, rs, 2, 3, cs, adpt_num_iter=3, adpt_mesh=2, adpt_fac=1).items():
        out['random_' + k] = v
    s2 = ref_system_from_arrays(wb, models.config_system(2, small=True))
    s2.do_ws_dist(mp_grid=3)
    EF2 = np.linspace(-1.5, 1.5, 31)
    out['EF2'] = EF2
    cs = {'ahc': calc.static.AHC(Efermi=EF2), 'bcd': calc.static.BerryDipole_FermiSea(Efermi=EF2)}
    for k, v in run_ref_adaptive(wb, s2, 2, [3, 4, 2], cs, adpt_num_iter=2, adpt_mesh=[2, 1, 3],
                                 adpt_fac=2).items():
        out['c2_' + k] = v
    # the tetrahedron method on refined K-points (their corners follow each K-point's cell)
    cs = {'ahc': calc.static.AHC(Efermi=EF, tetra=True), 'dos': calc.static.DOS(Efermi=EF, tetra=True)}
    for k, v in run_ref_adaptive(wb, rs, 2, 3, cs, adpt_num_iter=2, adpt_mesh=2, adpt_fac=1).items():
        out['tetra_random_' + k] = v
    np.savez_compressed(os.path.join(HERE, 'refine_ref.npz'), **out)


if __name__ == '__main__':
    root = sys.argv[1] if len(sys.argv) > 1 else '/root/reference'
    section = sys.argv[2] if len(sys.argv) > 2 else None
    if section in ('random', 'tetra', 'refine', 'dynamic', 'static', 'products'):  # one section only
        wb = setup_reference(root)
        from wannierberri.system.system_R import System_R
        rs = System_R.from_npz(path=os.path.join(root, 'tests', 'data', 'random'), legacy=True)
        if section == 'random':
            random_fixtures(root)
        else:
            {'tetra': tetra_fixtures, 'refine': refine_fixtures, 'dynamic': dynamic_fixtures,
             'static': static_fixtures, 'products': products_fixtures}[section](wb, rs)
    else:
        main(root)
