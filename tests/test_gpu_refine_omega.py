"""GPU test of the refinement around the largest Berry curvatures (wbgpu.run_refine_omega):
refining every k-point (top = 1, then mesh^3 in a second round) must give the grid with mesh times more points per axis, shifted
by -(mesh - 1) / (2 N mesh), evaluated directly; two rounds give mesh^2 times more.  This checks
the sub-grid phase tables (a k-step other than 1/NKFFT), the weights and the subtraction of the
refined points' own values.  A partial refinement moves the result from the coarse grid toward the
fine one."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import wbgpu  # noqa: E402
from wbgpu import engine, models, system as wsys  # noqa: E402
from wbgpu.run import _evaluate_blocks, run_refine_omega  # noqa: E402

C = wbgpu.calculators


def _system():
    s = wsys.System_R.from_dict(models.config_system(2, small=True))
    s.do_ws_dist(3)
    return s


def _calcs():
    ef = np.linspace(-1.0, 1.0, 41)
    return {'ahc': C.AHC(Efermi=ef), 'dos': C.DOS(Efermi=ef), 'bcd': C.BerryDipole_FermiSea(Efermi=ef)}


def _fine(s, dev, div, fft, M, precision):
    g = wbgpu.Grid(s, NKdiv=div, NKFFT=tuple(np.array(fft) * M))
    N = np.array(div) * np.array(fft)
    shifts = g.block_shifts() - (M - 1) / (2.0 * N * M)
    cs = _calcs()
    q = set()
    for c in cs.values():
        c.reset(dev.device)
        q |= c.quantities(s)
    _evaluate_blocks(dev, s, shifts, g.FFT, None, cs, q, precision, False)
    return {k: c.result(s.cell_volume, g.nk_per_block, 1.0 / g.nblocks) for k, c in cs.items()}


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-10), ('mixed', 1e-6)])
@pytest.mark.parametrize("rounds", [1, 2])
def test_refine_everything_equals_finer_grid(precision, tol, rounds):
    s = _system()
    dev = engine.DeviceSystem(s)
    div, fft, M = (2, 1, 2), (3, 2, 2), 2
    # every point of every round: the second round refines mesh^3 times the grid's points
    got = run_refine_omega(s, wbgpu.Grid(s, NKdiv=div, NKFFT=fft), _calcs(), precision=precision, rounds=rounds,
                           top=float(M ** 3) ** (rounds - 1), mesh=M, dev_system=dev)
    ref = _fine(s, dev, div, fft, M ** rounds, precision)
    for k in ref:
        a, b = got[k].data, ref[k].data
        assert np.max(np.abs(a - b)) <= tol * np.max(np.abs(b)), (k, np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_partial_refinement_between_coarse_and_fine():
    """top = 0.5: the refined result differs from the coarse one and the selected points are those
    of the largest |Omega|, so it is closer to the fine grid in the AHC than the coarse grid is."""
    s = _system()
    dev = engine.DeviceSystem(s)
    div, fft, M = (2, 2, 2), (3, 3, 3), 4
    g = wbgpu.Grid(s, NKdiv=div, NKFFT=fft)
    coarse = wbgpu.run(s, g, _calcs(), precision='fp64', dev_system=dev)
    part = run_refine_omega(s, g, _calcs(), precision='fp64', rounds=1, top=0.5, mesh=M, dev_system=dev)
    fine = _fine(s, dev, div, fft, M, 'fp64')
    dc = np.abs(coarse['ahc'].data - fine['ahc'].data).sum()
    dp = np.abs(part['ahc'].data - fine['ahc'].data).sum()
    assert np.abs(part['ahc'].data - coarse['ahc'].data).max() > 0
    assert dp < dc


def test_served_refinement_equals_run():
    """The Server's rounds of a refinement around |Omega| (two requests at once) give
    run_refine_omega's results."""
    s = _system()
    dev = engine.DeviceSystem(s)
    g = wbgpu.Grid(s, NKdiv=(2, 2, 1), NKFFT=(3, 3, 4))
    ref = run_refine_omega(s, g, _calcs(), precision='mixed', rounds=2, top=0.05, mesh=4, dev_system=dev)
    srv = wbgpu.Server(precision='mixed', max_active=2)
    srv.add_system(0, s)
    tickets = [srv.submit(0, g, _calcs(), refine_omega=2, refine_top=0.05, refine_mesh=4) for _ in range(2)]
    srv.run_until_idle()
    for t in tickets:
        got = t.wait(60)
        for k in ref:
            a, b = got[k].data, ref[k].data
            assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b)), k
