"""Host logic of the autotuner and of the CUDA-graph batch cache (no GPU needed).

* The library's launch-shape table: candidate lists for every num_wann, rejection of values
  the kernels do not accept, set / get / reset.
* coordinate_descent picks the fastest candidate per parameter; the JSON cache round-trips.
* engine.band_data_graphed's policy, with band_data and the CUDA graph replaced by recorders:
  first batch of a shape plain, second captured (plain run on the fixed phase inputs, then
  the capture), later ones replayed with the batch's phase tables copied into the inputs; a
  workspace reallocation or another system drops the graph.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from wbgpu import _lib, autotune, engine  # noqa: E402


@pytest.fixture(autouse=True)
def _reset_table():
    yield
    autotune.reset()


def test_candidates_cover_every_nw():
    for nw in range(1, 129):
        for variant in range(5):
            for p in autotune.EIGH_PARAMS:
                c = autotune.candidates(p, nw, variant)
                assert c and c == sorted(c) and all(v & (v - 1) == 0 for v in c), (nw, variant, p)
        for fp64 in (0, 1):
            kp = autotune.candidates(autotune.ROTATE_KPOINTS, nw, fp64)
            assert bool(kp) == (nw % 4 == 0 and 8 <= nw <= 64), (nw, fp64, kp)
            eng = autotune.candidates(autotune.ROTATE_ENGINE, nw, fp64)
            assert eng == ([1, 2, 3] if (nw == 32 and fp64 == 0) else [])


def test_set_get_reject():
    nw, variant = 32, 3
    for p in autotune.EIGH_PARAMS:
        cands = autotune.candidates(p, nw, variant)
        for v in cands:
            autotune.set_value(p, nw, variant, v)
            assert autotune.get_value(p, nw, variant) == v
        bad = [v for v in (3, 5, 512, 1024) if v not in cands]
        for v in bad:
            with pytest.raises(ValueError):
                autotune.set_value(p, nw, variant, v)
        assert autotune.get_value(p, nw, variant) == cands[-1]  # a rejected value leaves the entry
        autotune.set_value(p, nw, variant, 0)
        assert autotune.get_value(p, nw, variant) == 0
    with pytest.raises(ValueError):
        autotune.set_value(autotune.ROTATE_ENGINE, 16, 0, 1)  # no tensor-core rotation at nw = 16
    for args in [(-1, 8, 1, 0), (6, 8, 1, 0), (0, 0, 1, 0), (0, 129, 1, 0), (0, 8, 6, 0), (0, 8, 1, -1)]:
        with pytest.raises(ValueError):
            autotune.set_value(*args)
    autotune.set_value(autotune.EIGH_QL_BLOCK, 8, 1, 64)
    autotune.reset([8])
    assert autotune.get_value(autotune.EIGH_QL_BLOCK, 8, 1) == 0


def test_kubo_engine_entry():
    """The Kubo engine is one process-wide entry (variant 0, nw 1): 1 tensor cores, 2 CUDA cores."""
    assert autotune.candidates(autotune.KUBO_ENGINE, 1, 0) == [1, 2]
    assert autotune.candidates(autotune.KUBO_ENGINE, 2, 0) == []
    for bad in [(1, 0, 3), (2, 0, 1), (1, 1, 1)]:
        with pytest.raises(ValueError):
            autotune.set_value(autotune.KUBO_ENGINE, *bad)
    autotune.set_value(autotune.KUBO_ENGINE, 1, 0, 2)
    assert autotune.get_value(autotune.KUBO_ENGINE, 1, 0) == 2
    autotune.reset([1])
    assert autotune.get_value(autotune.KUBO_ENGINE, 1, 0) == 0


def test_exports_declared():
    lib = _lib.load()
    for name in ('wbg_tune_candidates', 'wbg_tune_set', 'wbg_tune_get'):
        assert hasattr(lib, name) and name in _lib.EXPORTS


def test_coordinate_descent():
    state = {}
    cost = {('a', 1): 3.0, ('a', 2): 1.0, ('a', 4): 2.0, ('b', 8): 5.0, ('b', 16): 5.0}

    def apply(p, v):
        state[p] = v

    def timing():
        return cost[('a', state['a'])] + (cost[('b', state['b'])] if 'b' in state else 0.0)

    best, times = autotune.coordinate_descent({'a': [1, 2, 4], 'b': [8, 16], 'c': []}, timing, apply)
    assert best == {'a': 2, 'b': 8} and state == {'a': 2, 'b': 8}  # tie on b: first measured
    assert times['a'] == {1: 3.0, 2: 1.0, 4: 2.0} and 'c' not in times


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / 'sub' / 'tune.json')
    assert autotune.load_cache(path) == {}
    data = {'GB300|abi1|nw32|mixed': {'eigh_tridiag_group': 4, 'eigh_ql_block': 64, 'rotate_engine': 2}}
    autotune.save_cache(data, path)
    assert autotune.load_cache(path) == data
    autotune.apply_entry(data['GB300|abi1|nw32|mixed'], 32, 'mixed')
    v = autotune.eigh_variant(autotune.PRECISION_VARIANTS['mixed'][0])
    assert autotune.get_value(autotune.EIGH_TRIDIAG_GROUP, 32, v) == 4
    assert autotune.get_value(autotune.EIGH_QL_BLOCK, 32, v) == 64
    assert autotune.get_value(autotune.ROTATE_ENGINE, 32, 0) == 2
    assert autotune.get_value(autotune.EIGH_TRIDIAG_GROUP, 32, 1) == 0  # FP64 variant untouched
    with open(path, 'w') as f:
        f.write('not json')
    assert autotune.load_cache(path) == {}


class _FakeDev:
    def __init__(self):
        iR = np.array([[a, b, c] for a in range(-1, 2) for b in range(-1, 2) for c in range(-2, 3)])
        self.geom = engine.RGeometry(iR)
        self._ws = engine.Workspace('cpu')

    def workspace(self):
        return self._ws


class _Recorder:
    """Stands in for engine.band_data and for the CUDA graph calls."""

    def __init__(self, monkeypatch):
        self.calls = []  # (phases, block_start, nb, captured)
        self.capturing = False
        self.replays = 0
        rec = self

        class Graph:
            def replay(self):
                rec.replays += 1

        class GraphCtx:
            def __init__(self, graph, capture_error_mode='global'):
                assert capture_error_mode == 'relaxed'

            def __enter__(self):
                rec.capturing = True

            def __exit__(self, *a):
                rec.capturing = False

        def band_data(dev, dKs, NKFFT, quantities, precision='fp64', phases=None, block_start=0, ws=None):
            self.calls.append((phases, block_start, len(dKs), self.capturing))
            return engine.BandData(None, None, None, {}, len(dKs), int(np.prod(NKFFT)), 4, precision == 'fp64')

        monkeypatch.setattr(engine, 'band_data', band_data)
        monkeypatch.setattr(torch.cuda, 'CUDAGraph', Graph)
        monkeypatch.setattr(torch.cuda, 'graph', GraphCtx)


def _grid_tables(dev, shifts, NKFFT):
    return {engine.PREC_FP64: [torch.from_numpy(t) for t in dev.geom.phases(shifts, NKFFT)]}


def test_graph_policy_grid_tables(monkeypatch):
    rec = _Recorder(monkeypatch)
    dev = _FakeDev()
    NKFFT = (3, 2, 4)
    shifts = np.random.default_rng(0).uniform(0, 0.3, (8, 3))
    ph = _grid_tables(dev, shifts, NKFFT)
    q = {'V', 'A'}
    run = lambda i0, nb=2, d=dev: engine.band_data_graphed(d, shifts[i0:i0 + nb], NKFFT, q, 'fp64', phases=ph,
                                                          block_start=i0)
    run(0)  # first of its shape: plain launches on the grid tables
    assert rec.calls == [(ph, 0, 2, False)]
    run(2)  # second: plain run on the fixed inputs, then the capture
    assert [(c[1], c[2], c[3]) for c in rec.calls[1:]] == [(0, 2, False), (0, 2, True)]
    tabs = rec.calls[1][0]
    assert tabs is rec.calls[2][0] and tabs is not ph
    for d in range(3):
        assert torch.equal(tabs[engine.PREC_FP64][d], ph[engine.PREC_FP64][d][2:4])
    run(6)  # replay: no band_data call, the batch's tables in the inputs
    assert len(rec.calls) == 3 and rec.replays == 1
    for d in range(3):
        assert torch.equal(tabs[engine.PREC_FP64][d], ph[engine.PREC_FP64][d][6:8])
    key = (NKFFT, 2, frozenset(q), 'fp64')
    assert dev.workspace().graphs[key].replays == 1
    run(5, nb=3)  # another shape: plain
    assert rec.calls[-1] == (ph, 5, 3, False)
    # a reallocated buffer drops the graph: captured again at the next batch of the shape
    dev.workspace().buffer('grown', (4096,), torch.uint8)
    n = len(rec.calls)
    run(4)
    assert [c[3] for c in rec.calls[n:]] == [False, True] and rec.replays == 1
    run(0)
    assert rec.replays == 2
    # another system on the same workspace: plain first, its own capture second
    dev2 = _FakeDev()
    dev2._ws = dev.workspace()
    dev2.geom = dev.geom
    n = len(rec.calls)
    run(0, d=dev2)
    assert [c[3] for c in rec.calls[n:]] == [False]
    run(2, d=dev2)
    assert [c[3] for c in rec.calls[n:]] == [False, False, True]
    assert dev.workspace().graphs[key].dev is dev2


def test_graph_policy_host_tables_mixed(monkeypatch):
    rec = _Recorder(monkeypatch)
    dev = _FakeDev()
    NKFFT = (2, 3, 2)
    rng = np.random.default_rng(1)
    q = {'V'}
    batches = [rng.uniform(-0.5, 0.5, (3, 3)) for _ in range(4)]
    for dKs in batches:
        engine.band_data_graphed(dev, dKs, NKFFT, q, 'mixed')
    assert [c[3] for c in rec.calls] == [False, False, True] and rec.replays == 2
    tabs = rec.calls[1][0]
    assert set(tabs) == {engine.PREC_DF64, engine.PREC_FP32S}
    host = dev.geom.phases(batches[-1], NKFFT)
    for d in range(3):
        assert np.array_equal(tabs[engine.PREC_DF64][d].numpy(), engine._df64_pairs(host[d]))
        assert np.array_equal(tabs[engine.PREC_FP32S][d].numpy(), host[d].astype(np.complex64))
    # energies-only batches need the double-float tables alone
    rec2 = _Recorder(monkeypatch)
    for dKs in batches[:2]:
        engine.band_data_graphed(dev, dKs, NKFFT, set(), 'mixed')
    assert set(rec2.calls[1][0]) == {engine.PREC_DF64}


def test_graph_skipped_under_stage_timer(monkeypatch):
    rec = _Recorder(monkeypatch)
    dev = _FakeDev()
    engine.set_timer(object())
    try:
        for _ in range(3):
            engine.band_data_graphed(dev, np.zeros((1, 3)), (2, 2, 2), {'V'}, 'fp64')
    finally:
        engine.set_timer(None)
    assert [c[3] for c in rec.calls] == [False] * 3 and rec.replays == 0


def test_graph_capture_only_when_replayed(monkeypatch):
    rec = _Recorder(monkeypatch)
    dev = _FakeDev()
    NKFFT = (2, 2, 2)
    dKs = np.zeros((2, 3))
    for more in (True, False, False):  # the second batch would be captured, but nothing follows it
        engine.band_data_graphed(dev, dKs, NKFFT, {'V'}, 'fp64', more=more)
    assert [c[3] for c in rec.calls] == [False, False, False] and not dev.workspace().graphs
    engine.band_data_graphed(dev, dKs, NKFFT, {'V'}, 'fp64', more=True)  # now captured
    engine.band_data_graphed(dev, dKs, NKFFT, {'V'}, 'fp64', more=False)  # an existing graph replays
    assert [c[3] for c in rec.calls[3:]] == [False, True] and rec.replays == 1


def test_capture_hints_of_run_and_server():
    from wbgpu.run import more_batches_of_size
    from wbgpu.serve import later_batch_of_size
    # 8 blocks in batches of 3: 3, 3, 2 -> only the first full batch is followed by another of its size
    assert [more_batches_of_size(8, 3, i0) for i0 in (0, 3, 6)] == [True, False, False]
    assert [more_batches_of_size(8, 2, i0) for i0 in (0, 2, 4, 6)] == [True, True, True, False]
    assert more_batches_of_size(1, 4, 0) is False
    batches = [np.arange(0, 2), np.arange(2, 4), np.arange(4, 5)]
    assert later_batch_of_size(batches, 1, 2) and not later_batch_of_size(batches, 2, 2)
    assert later_batch_of_size(batches, 2, 1) and not later_batch_of_size(batches, 3, 1)
