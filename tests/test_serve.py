"""Continuous batching on the GPU: every request's result is the same alone (run()) and in the
mix of concurrent requests on other systems -- bit for bit: every per-k-point computation is
independent of how the blocks are batched, the Kubo pair records are stored in pair order, and
every histogram and frequency sum is accumulated in order-independent fixed point."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import wbgpu  # noqa: E402
from wbgpu import models, system as wsys  # noqa: E402
from wbgpu.calculators import AHC, Morb, OpticalConductivity, BerryDipole_FermiSea  # noqa: E402


def _systems():
    c1 = wsys.System_R.from_dict(models.config_system(1))
    c2 = wsys.System_R.from_dict(models.config_system(2, small=True))
    c2.do_ws_dist(3)
    big = wsys.System_R.from_dict(models.random_tb(32, 1, models.triclinic_lattice(np.random.default_rng(9)), 1.5, 932,
                                                   centers='random', keys=('Ham', 'AA', 'BB', 'CC')))
    return {'c1': c1, 'c2': c2, 'nw32': big}


EF = np.linspace(-1, 1, 41)


def _requests():
    return [('c1', 4, 4, lambda: {'ahc': AHC(Efermi=EF)}),
            ('nw32', 2, 6, lambda: {'ahc': AHC(Efermi=EF), 'morb': Morb(Efermi=EF)}),
            ('c2', 3, 4, lambda: {'opt': OpticalConductivity(Efermi=EF[::10], omega=np.linspace(0.1, 2, 8))}),
            ('c1', 2, 8, lambda: {'bcd': BerryDipole_FermiSea(Efermi=EF)}),
            ('nw32', 1, 8, lambda: {'ahc': AHC(Efermi=EF)})]


def _close(a, b):
    for k in b:
        x, y = a[k].data, b[k].data
        assert np.array_equal(x, y), (k, np.abs(x - y).max())


@pytest.mark.parametrize("precision", ['mixed', 'fp64'])
@pytest.mark.parametrize("budget", [150 << 30, 1])
def test_results_same_alone_and_in_the_mix(precision, budget):
    systems = _systems()
    srv = wbgpu.Server(precision=precision, hbm_budget=budget, max_active=3)
    for key, s in systems.items():
        srv.add_system(key, s)
    tickets, alone = [], []
    for key, nkdiv, nkfft, mk in _requests():
        s = systems[key]
        grid = wbgpu.Grid(s, NKdiv=nkdiv, NKFFT=nkfft)
        tickets.append(srv.submit(key, grid, mk()))
        alone.append(wbgpu.run(s, grid, mk(), precision=precision))
    srv.run_until_idle()
    for t, ref in zip(tickets, alone):
        _close(t.wait(), ref)
    st = srv.stats()
    assert st['requests'] == len(tickets) and st['p99_ms'] >= st['p50_ms'] > 0


def test_background_thread_and_block_subsets():
    """Requests submitted while others run (scheduler thread); block subsets weight like run()."""
    systems = _systems()
    s = systems['nw32']
    grid = wbgpu.Grid(s, NKdiv=3, NKFFT=4)
    with wbgpu.Server(precision='mixed', max_active=2) as srv:
        srv.add_system('a', s)
        srv.add_system('b', systems['c1'])
        t1 = srv.submit('a', grid, {'ahc': AHC(Efermi=EF)}, blocks=[0, 5, 6, 7, 20])
        t2 = srv.submit('b', wbgpu.Grid(systems['c1'], NKdiv=3, NKFFT=4), {'ahc': AHC(Efermi=EF)})
        t3 = srv.submit('a', grid, {'ahc': AHC(Efermi=EF)}, blocks=[1, 2])
        r1, r2, r3 = t1.wait(60), t2.wait(60), t3.wait(60)
    _close(r1, wbgpu.run(s, grid, {'ahc': AHC(Efermi=EF)}, precision='mixed', blocks=[0, 5, 6, 7, 20]))
    _close(r3, wbgpu.run(s, grid, {'ahc': AHC(Efermi=EF)}, precision='mixed', blocks=[1, 2]))
    _close(r2, wbgpu.run(systems['c1'], wbgpu.Grid(systems['c1'], NKdiv=3, NKFFT=4), {'ahc': AHC(Efermi=EF)},
                         precision='mixed'))


def test_unknown_system_rejected():
    srv = wbgpu.Server()
    with pytest.raises(ValueError):
        srv.submit('nope', None, {})


def test_run_many_matches_run():
    systems = _systems()
    jobs = [(systems[k], wbgpu.Grid(systems[k], NKdiv=2, NKFFT=4), {'ahc': AHC(Efermi=EF)}) for k in ('c1', 'nw32', 'c2')]
    got = wbgpu.run_many(jobs, precision='mixed')
    for (s, g, _), r in zip(jobs, got):
        _close(r, wbgpu.run(s, g, {'ahc': AHC(Efermi=EF)}, precision='mixed'))
