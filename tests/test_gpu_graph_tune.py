"""CUDA-graph replay of stages 1-3 and the launch-shape autotuner, on the GPU through the C ABI.

* engine.band_data_graphed writes the same buffers as engine.band_data with the same kernels:
  E and the band-basis fields must be bit-identical, batch by batch (grid phase tables and
  host-built tables, FP64 and mixed precision, a tail batch of another size).
* run() / Server with cuda_graph=True against the plain launches: 1e-10 relative (only the
  order of the FP64 histogram atomics differs between two runs).
* Every launch shape the autotuner may select: eigensolver E and U bit-identical to the
  built-in shapes, tiled rotation bit-identical; the rotation engine (tensor cores / CUDA
  cores at nw = 32, FP32) within 2e-6 of the FP64 rotation.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import wbgpu  # noqa: E402
from wbgpu import autotune, engine, models, system as wsys  # noqa: E402
from wbgpu.calculators import AHC, Morb  # noqa: E402

EF = np.linspace(-1.5, 1.5, 61)


@pytest.fixture(autouse=True)
def _table_reset():
    yield
    autotune.reset()


@pytest.fixture(scope="module")
def systems():
    c1 = wsys.System_R.from_dict(models.config_system(1))
    nw32 = wsys.System_R.from_dict(models.random_tb(32, 1, models.triclinic_lattice(np.random.default_rng(5)), 1.5,
                                                    532, centers='random', keys=('Ham', 'AA', 'BB', 'CC')))
    return {'c1': c1, 'nw32': nw32}


def _snapshot(bd):
    """E and Xbar of a batch; the diagonal-only fields (rotA for Omega, quantity 'Od') are
    rotated only on their diagonal, so their off-diagonal entries are left out."""
    X = None if bd.Xbar is None else bd.Xbar.cpu().numpy().copy()
    if X is not None and 'Od' in bd.index and 'O' not in bd.index:
        i = bd.index['Od']
        X[:, i:i + 3, ~np.eye(bd.nw, dtype=bool)] = 0
    return bd.E.cpu().numpy().copy(), X


@pytest.mark.parametrize("precision", ['fp64', 'mixed'])
@pytest.mark.parametrize("name", ['c1', 'nw32'])
def test_graphed_band_data_bit_identical(systems, name, precision):
    s = systems[name]
    dev = engine.DeviceSystem(s)
    grid = wbgpu.Grid(s, NKdiv=(2, 2, 2), NKFFT=(4, 3, 4))
    shifts = grid.block_shifts()
    q = {'V', 'A', 'Od', 'W'} if precision == 'fp64' else {'V', 'A', 'Od'}
    precs = [engine.PREC_FP64] if precision == 'fp64' else [engine.PREC_DF64, engine.PREC_FP32S]
    phases = {p: dev.grid_phases(shifts, grid.FFT, p) for p in precs}
    ws_plain, ws_graph = engine.Workspace('cuda'), engine.Workspace('cuda')
    for i0, nb in [(0, 2), (2, 2), (4, 2), (6, 2), (0, 2), (5, 3)]:
        dKs = shifts[i0:i0 + nb]
        a = _snapshot(engine.band_data(dev, dKs, grid.FFT, q, precision, phases=phases, block_start=i0, ws=ws_plain))
        b = _snapshot(engine.band_data_graphed(dev, dKs, grid.FFT, q, precision, phases=phases, block_start=i0,
                                               ws=ws_graph))
        assert np.array_equal(a[0], b[0]), (i0, nb)
        assert np.array_equal(a[1], b[1]), (i0, nb)
    ent = ws_graph.graphs[(tuple(grid.FFT), 2, frozenset(q), precision)]
    assert ent.replays == 3  # batch (0, 2) plain, (2, 2) captured, (4, 2), (6, 2), (0, 2) replayed
    # tables built on the host (no grid tables): shifts off the grid
    rng = np.random.default_rng(3)
    for _ in range(3):
        dKs = rng.uniform(-0.5, 0.5, (2, 3)) / grid.FFT
        a = _snapshot(engine.band_data(dev, dKs, grid.FFT, q, precision, ws=ws_plain))
        b = _snapshot(engine.band_data_graphed(dev, dKs, grid.FFT, q, precision, ws=ws_graph))
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    engine.check_flag(engine.band_data(dev, shifts[:1], grid.FFT, q, precision, ws=ws_plain))


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("precision", ['fp64', 'mixed'])
def test_run_cuda_graph(systems, precision):
    s = systems['nw32']
    grid = wbgpu.Grid(s, NKdiv=(2, 2, 2), NKFFT=4)
    mk = lambda: {'ahc': AHC(Efermi=EF), 'morb': Morb(Efermi=EF)}
    ref = wbgpu.run(s, grid, mk(), precision=precision, blocks_per_batch=3)
    dev = engine.DeviceSystem(s)
    got = wbgpu.run(s, grid, mk(), precision=precision, blocks_per_batch=3, cuda_graph=True, dev_system=dev)
    got2 = wbgpu.run(s, grid, mk(), precision=precision, blocks_per_batch=3, cuda_graph=True, dev_system=dev)
    for k in ref:
        assert _rel(got[k].data, ref[k].data) < 1e-10, k
        assert _rel(got2[k].data, ref[k].data) < 1e-10, k
    assert any(e.replays > 0 for e in dev.workspace().graphs.values())


def test_server_cuda_graph(systems):
    grid = wbgpu.Grid(systems['c1'], NKdiv=(3, 2, 2), NKFFT=4)
    ref = {k: wbgpu.run(systems[k], grid, {'ahc': AHC(Efermi=EF)}, precision='mixed', blocks_per_batch=2)
           for k in systems}
    srv = wbgpu.Server(precision='mixed', max_active=2, max_kpoints=2 * 64, cuda_graph=True)
    for k, s in systems.items():
        srv.add_system(k, s)
    tickets = [(k, srv.submit(k, grid, {'ahc': AHC(Efermi=EF)})) for k in systems for _ in range(2)]
    srv.run_until_idle()
    for k, t in tickets:
        assert _rel(t.wait()['ahc'].data, ref[k]['ahc'].data) < 1e-10, k


def _hermitian(nk, nw, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw))
    return 0.5 * (A + np.conj(np.swapaxes(A, 1, 2)))


@pytest.mark.parametrize("mode", [1, 3])
@pytest.mark.parametrize("nw", [4, 8, 32, 96])
def test_eigh_tuned_shapes_bit_identical(nw, mode):
    nk = 777  # not a multiple of any group size: every launch has a partial last block
    H = _hermitian(nk, nw, 100 + nw)
    Hd = torch.from_numpy(engine._df64_pairs(H) if mode == 3 else H).cuda()

    def solve():
        E, U, flag = engine.eigh(Hd, nw * nw, nw, nk, mode=mode)
        assert int(flag.item()) == 0
        return E.cpu().numpy(), U.cpu().numpy()

    E0, U0 = solve()
    for p in autotune.EIGH_PARAMS:
        for v in autotune.candidates(p, nw, mode & 3):
            autotune.set_value(p, nw, mode & 3, v)
            E1, U1 = solve()
            assert np.array_equal(E0, E1) and np.array_equal(U0, U1), (autotune.PARAM_NAMES[p], v)
        autotune.set_value(p, nw, mode & 3, 0)


def test_rotate_tuned_shapes():
    rng = np.random.default_rng(7)
    for nw, fp64 in [(16, 0), (16, 1), (32, 1), (48, 0)]:
        nk, nf = 301, 3
        cdt = torch.complex128 if fp64 else torch.complex64
        U = torch.from_numpy(rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw))).cuda().to(cdt)
        X = torch.from_numpy(rng.standard_normal((nk, nf, nw, nw)) + 1j * rng.standard_normal((nk, nf, nw, nw))
                             ).cuda().to(cdt)
        sel, herm = list(range(nf)), [0, 1, 2]
        base = engine.rotate(U, X, nf, sel, herm, nw, nk, bool(fp64))[0].cpu().numpy()
        cands = autotune.candidates(autotune.ROTATE_KPOINTS, nw, fp64)
        assert cands
        for v in cands:
            autotune.set_value(autotune.ROTATE_KPOINTS, nw, fp64, v)
            got = engine.rotate(U, X, nf, sel, herm, nw, nk, bool(fp64))[0].cpu().numpy()
            # herm = 2 writes at least the diagonal: compare the diagonal there, everything elsewhere
            assert np.array_equal(got[:, :2], base[:, :2]), (nw, fp64, v)
            assert np.array_equal(np.diagonal(got[:, 2], axis1=-2, axis2=-1),
                                  np.diagonal(base[:, 2], axis1=-2, axis2=-1)), (nw, fp64, v)
        autotune.set_value(autotune.ROTATE_KPOINTS, nw, fp64, 0)


def test_rotate_engine_choice():
    nw, nk, nf = 32, 257, 4
    rng = np.random.default_rng(11)
    Q = np.linalg.qr(rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw)))[0]
    Xh = rng.standard_normal((nk, nf, nw, nw)) + 1j * rng.standard_normal((nk, nf, nw, nw))
    sel, herm = list(range(nf)), [0, 1, 0, 1]
    ref = engine.rotate(torch.from_numpy(Q).cuda(), torch.from_numpy(Xh).cuda(), nf, sel, herm, nw, nk,
                        True)[0].cpu().numpy()
    U32, X32 = torch.from_numpy(Q).cuda().to(torch.complex64), torch.from_numpy(Xh).cuda().to(torch.complex64)
    assert autotune.candidates(autotune.ROTATE_ENGINE, nw, 0) == [1, 2, 3]
    outs = []
    for v in (1, 2, 3):
        autotune.set_value(autotune.ROTATE_ENGINE, nw, 0, v)
        outs.append(engine.rotate(U32, X32, nf, sel, herm, nw, nk, False)[0].cpu().numpy())
        assert _rel(outs[-1], ref) < 2e-6, v
    autotune.set_value(autotune.ROTATE_ENGINE, nw, 0, 0)
    assert not np.array_equal(outs[0], outs[1])  # tensor and CUDA cores really ran
    assert np.array_equal(outs[0], outs[2])  # the two tensor-core kernels do the same arithmetic


def test_autotune_ensure_and_run(systems, tmp_path, monkeypatch):
    monkeypatch.setenv('WBGPU_TUNE_CACHE', str(tmp_path / 'tune.json'))
    s = systems['c1']
    entry = autotune.ensure(s.num_wann, 'fp64')
    assert set(entry) <= set(autotune.PARAM_NAMES.values()) and entry
    for name, v in entry.items():
        p = {n: k for k, n in autotune.PARAM_NAMES.items()}[name]
        variant = 1
        assert autotune.get_value(p, s.num_wann, variant) == v
    autotune.reset()
    again = autotune.ensure(s.num_wann, 'fp64')  # from the cache file, no measurement
    assert again == entry
    grid = wbgpu.Grid(s, NKdiv=2, NKFFT=4)
    autotune.reset()
    ref = wbgpu.run(s, grid, {'ahc': AHC(Efermi=EF)}, precision='fp64')
    got = wbgpu.run(s, grid, {'ahc': AHC(Efermi=EF)}, precision='fp64', autotune=True)
    assert _rel(got['ahc'].data, ref['ahc'].data) < 1e-10
    e32, t32 = autotune.tune_eigh(32, 3, nk=4096, reps=1)
    assert set(e32) == {'eigh_tridiag_group', 'eigh_ql_block', 'eigh_vectors_group'}
    for name, times in t32.items():
        assert min(times.values()) > 0
