"""Parity at the benchmark configurations: the full models the benchmark runs, on reduced grids,
through run() against the oracle, in both precisions.

* nw = 32 triclinic model, R in [-4,4]^3, MDRS (mp_grid 9, ~1275 R-vectors): AHC, Morb and the
  Berry-curvature dipole at 1001 Fermi levels on one 12^3 FFT block -- the benchmarked path: the
  double-float eigensolver on lower triangles, the tensor-core rotation (nw = 32, FP32) and the
  column Omega kernel.
* nw = 96 spinor model with SOC blocks, R in [-5,5]^3: AHC and the Kubo optical conductivity
  (11 levels x 400 frequencies, Lorentzian 0.05 eV) on one 4^3 block; the AHC again on an 8^3 block.

Tolerances (max over levels and components / max |result|): FP64 path 1e-9; mixed path 1e-6.
The oracle runs in spawned processes while the GPU works.
"""
import multiprocessing as mp
import os
import tempfile

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import wbgpu  # noqa: E402
from wbgpu import models, system as wsys  # noqa: E402

EF1001 = np.linspace(-2, 2, 1001)
EF11 = np.linspace(-1, 1, 11)
OMEGA = np.linspace(0, 4, 400)


def _oracle_job(args):
    """One oracle run() in a spawned process: (key, {calculator: data})."""
    key, path, NKdiv, NKFFT, names = args
    from oracle import wb_oracle as O
    f = np.load(path)
    XX = {k[3:]: f[k] for k in f.files if k.startswith('XX_')}
    o = O.RSystem(f['real_lattice'], f['iRvec'], f['wcc'], XX)
    calcs = {}
    for n in names:
        if n == 'ahc1001':
            calcs[n] = O.AHC(Efermi=EF1001)
        elif n == 'morb':
            calcs[n] = O.Morb(Efermi=EF1001)
        elif n == 'bcd':
            calcs[n] = O.BerryDipole_FermiSea(Efermi=EF1001)
        elif n == 'ahc11':
            calcs[n] = O.AHC(Efermi=EF11)
        elif n == 'opt':
            calcs[n] = O.OpticalConductivity(Efermi=EF11, omega=OMEGA, smr_fixed_width=0.05)
    res = O.run(o, NKdiv, NKFFT, calcs)
    return key, {k: np.asarray(v.data) for k, v in res.items()}


def _save(s, keys):
    fd, path = tempfile.mkstemp(suffix='.npz', prefix='wbhead_')
    os.close(fd)
    np.savez(path, real_lattice=s.real_lattice, iRvec=s.iRvec, wcc=s.wannier_centers_cart,
             **{'XX_' + k: s.get_R_mat(k) for k in keys})
    return path


@pytest.fixture(scope="module")
def models_and_oracle():
    """The two benchmark models on the device and the oracle's results, computed asynchronously
    (one spawned process per job) while the tests run."""
    c2 = wsys.System_R.from_dict(models.config_system(2))
    c2.do_ws_dist(9, device='cuda')
    c3 = wsys.System_R.from_dict(models.config_system(3))
    p2, p3 = _save(c2, ('Ham', 'AA', 'BB', 'CC')), _save(c3, ('Ham', 'AA'))
    jobs = [('c2_ahc', p2, (1, 1, 1), (12, 12, 12), ['ahc1001']),
            ('c2_morb', p2, (1, 1, 1), (12, 12, 12), ['morb']),
            ('c2_bcd', p2, (1, 1, 1), (12, 12, 12), ['bcd']),
            ('c3_opt', p3, (1, 1, 1), (4, 4, 4), ['ahc11', 'opt']),
            ('c3_ahc8', p3, (1, 1, 1), (8, 8, 8), ['ahc11'])]
    pool = mp.get_context('spawn').Pool(min(len(jobs), os.cpu_count() or 1))
    pending = pool.map_async(_oracle_job, jobs)
    cache = {}

    def oracle(key):
        if not cache:
            cache.update(dict(pending.get(timeout=1800)))
            pool.close()
            for p in (p2, p3):
                os.unlink(p)
        return cache[key]

    yield c2, c3, oracle
    pool.terminate()


def maxrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-9), ('mixed', 1e-6)])
def test_nw32_mdrs_ahc_morb_bcd(models_and_oracle, precision, tol):
    c2, _, oracle = models_and_oracle
    C = wbgpu.calculators
    grid = wbgpu.Grid(c2, NKdiv=1, NKFFT=12)
    got = {'ahc1001': wbgpu.run(c2, grid, {'a': C.AHC(Efermi=EF1001)}, precision=precision)['a'].data,
           'morb': wbgpu.run(c2, grid, {'a': C.Morb(Efermi=EF1001)}, precision=precision)['a'].data,
           'bcd': wbgpu.run(c2, grid, {'a': C.BerryDipole_FermiSea(Efermi=EF1001)}, precision=precision)['a'].data}
    ref = {**oracle('c2_ahc'), **oracle('c2_morb'), **oracle('c2_bcd')}
    for key, g in got.items():
        assert g.shape == ref[key].shape, key
        assert maxrel(g, ref[key]) < tol, (key, precision, maxrel(g, ref[key]))


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-9), ('mixed', 1e-6)])
def test_nw96_spinor_kubo_and_ahc(models_and_oracle, precision, tol):
    _, c3, oracle = models_and_oracle
    C = wbgpu.calculators
    res = wbgpu.run(c3, wbgpu.Grid(c3, NKdiv=1, NKFFT=4),
                    {'opt': C.OpticalConductivity(Efermi=EF11, omega=OMEGA, smr_fixed_width=0.05),
                     'ahc11': C.AHC(Efermi=EF11)}, precision=precision)
    ref = oracle('c3_opt')
    for key in ('opt', 'ahc11'):
        assert maxrel(res[key].data, ref[key]) < tol, (key, precision, maxrel(res[key].data, ref[key]))
    res8 = wbgpu.run(c3, wbgpu.Grid(c3, NKdiv=1, NKFFT=8), {'ahc11': C.AHC(Efermi=EF11)}, precision=precision)
    ref8 = oracle('c3_ahc8')['ahc11']
    assert maxrel(res8['ahc11'].data, ref8) < tol, ('ahc 8^3', precision, maxrel(res8['ahc11'].data, ref8))
