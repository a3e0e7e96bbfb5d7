"""Failure isolation of the continuous-batching server, with the failures made on the host (no GPU
fault): a calculator that raises while its batch is issued, one that raises when its result is read,
a request for a system that was never added, and a ticket whose wait runs out.  The failing request
gets its error; every other request in the mix finishes with the same bits as run() alone."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import wbgpu  # noqa: E402
from wbgpu import models, system as wsys  # noqa: E402
from wbgpu.calculators import AHC  # noqa: E402

EF = np.linspace(-1, 1, 21)


class AccumulateFails(AHC):
    def accumulate(self, bd, system):
        raise RuntimeError("injected failure in accumulate")


class ResultFails(AHC):
    def result(self, *a, **k):
        raise RuntimeError("injected failure in result")


def _system():
    return wsys.System_R.from_dict(models.config_system(1))


@pytest.mark.parametrize("bad", [AccumulateFails, ResultFails])
def test_failing_request_fails_alone(bad):
    s = _system()
    grid = wbgpu.Grid(s, NKdiv=2, NKFFT=4)
    srv = wbgpu.Server(precision='mixed', max_active=3)
    srv.add_system('a', s)
    good = [srv.submit('a', grid, {'ahc': AHC(Efermi=EF)}) for _ in range(2)]
    broken = srv.submit('a', grid, {'ahc': bad(Efermi=EF)})
    good.append(srv.submit('a', grid, {'ahc': AHC(Efermi=EF)}))
    srv.run_until_idle()
    with pytest.raises(RuntimeError, match="injected"):
        broken.wait(1)
    ref = wbgpu.run(s, grid, {'ahc': AHC(Efermi=EF)}, precision='mixed')['ahc'].data
    for t in good:
        assert np.array_equal(t.wait(1)['ahc'].data, ref)
    assert srv.stats()['requests'] == 4


def test_unknown_system_and_wait_timeout():
    s = _system()
    grid = wbgpu.Grid(s, NKdiv=2, NKFFT=4)
    srv = wbgpu.Server(precision='mixed', max_active=2)
    srv.add_system('a', s)
    with pytest.raises(ValueError):
        srv.submit('missing', grid, {'ahc': AHC(Efermi=EF)})
    t = srv.submit('a', grid, {'ahc': AHC(Efermi=EF)})
    with pytest.raises(TimeoutError):  # no scheduler has run yet
        t.wait(0.01)
    srv.run_until_idle()
    assert t.wait(1)['ahc'].data.shape == (len(EF), 3)
