"""The mixed path's Kubo band sums on the tensor cores (kubo_tc, wbg_tune WBG_TUNE_KUBO_ENGINE 1, the
built-in choice) against the CUDA-core register-tiled GEMM (engine 2) and the oracle: the frequency
factor times the f_E-weighted pair records as a 3xTF32 complex GEMM per k-point
(calculators/dynamic.py:97-98).  Several frequency tiles (nOmega > 128), several column tiles
(27 components x 5 levels > 104 columns), Lorentzian and Gaussian smearing, every formula with 9 or 27
components; the output is bit-identical from run to run (fixed-point sums)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import wb_oracle as O  # noqa: E402
from wbgpu import autotune, models, system as wsys  # noqa: E402
import wbgpu  # noqa: E402

C = wbgpu.calculators


def _system():
    d = models.config_system(2, small=True)
    s = wsys.System_R.from_dict(d)
    s.do_ws_dist(3)
    return s


def _calcs(M, EF, om):
    pL = dict(Efermi=EF, omega=om, smr_fixed_width=0.1)
    pG = dict(Efermi=EF, omega=om, smr_fixed_width=0.15, smr_type='Gaussian', kBT=0.02)
    return {'opt_L': M.OpticalConductivity(**pL), 'opt_G': M.OpticalConductivity(**pG),
            'shift_L': M.ShiftCurrent(sc_eta=0.05, **pL), 'inj_G': M.InjectionCurrent(**pG)}


def _run(s, engine, EF, om, nk=(4, 5, 3)):
    autotune.set_value(autotune.KUBO_ENGINE, 1, 0, engine)
    try:
        return wbgpu.run(s, wbgpu.Grid(s, NKdiv=1, NKFFT=nk), _calcs(C, EF, om), precision='mixed')
    finally:
        autotune.set_value(autotune.KUBO_ENGINE, 1, 0, 0)


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_kubo_tc_vs_cuda_cores_and_oracle():
    s = _system()
    EF = np.linspace(-0.6, 0.6, 5)
    om = np.linspace(0.0, 3.0, 300)
    tc = _run(s, 1, EF, om)
    cc = _run(s, 2, EF, om)
    o = O.RSystem(s.real_lattice, s.iRvec, s.wannier_centers_cart, s._XX_R)
    ref = O.run(o, (1, 1, 1), (4, 5, 3), _calcs(O, EF, om))
    for q in tc:
        assert _rel(tc[q].data, cc[q].data) < 1e-6, (q, _rel(tc[q].data, cc[q].data))
        assert _rel(tc[q].data, ref[q].data) < 1e-6, (q, _rel(tc[q].data, ref[q].data))


def test_kubo_tc_deterministic():
    s = _system()
    EF = np.linspace(-0.6, 0.6, 3)
    om = np.linspace(0.0, 3.0, 150)
    a = _run(s, 1, EF, om, nk=(6, 6, 6))
    b = _run(s, 1, EF, om, nk=(6, 6, 6))
    for q in a:
        assert np.array_equal(a[q].data, b[q].data), q
