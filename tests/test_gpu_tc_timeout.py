"""Failure detection of the tensor-core rotation without a GPU fault: a wait that runs out records
WBG_DEVICE_FLAG_TC_TIMEOUT, the kernel drains its own products, frees its tensor memory and returns,
and the next call on the same context is correct.

* wbg_tc_wait_probe waits on an mbarrier phase that never completes, with a 1 ms bound.
* the rotation itself with a 0 ns bound: a block whose products are not done when it first looks
  gives up; afterwards, with the normal bound, the rotation is correct and unflagged.
* the tensor-core Kubo sums with a 0 ns bound, then the same run again with the normal bound.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from wbgpu import _lib, engine  # noqa: E402

DEFAULT_NS = 1_000_000_000


def _flags(clear=True):
    f = ctypes.c_uint(0)
    _lib.check(_lib.load().wbg_device_flags(ctypes.byref(f), int(clear)), "wbg_device_flags")
    return f.value


def _rotation_case(nk=4096, nF=9, seed=3):
    rng = np.random.default_rng(seed)
    nw = 32
    X = rng.standard_normal((nk, nF, nw, nw)) + 1j * rng.standard_normal((nk, nF, nw, nw))
    U = np.linalg.qr(rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw)))[0]
    return (torch.from_numpy(U).to(torch.complex64).cuda(), torch.from_numpy(X).to(torch.complex64).cuda(),
            torch.from_numpy(U).cuda(), torch.from_numpy(X).cuda())


def test_wait_probe_runs_out_and_flags():
    lib = _lib.load()
    _flags()
    res = torch.full((1,), 7, dtype=torch.int32, device='cuda')
    try:
        _lib.check(lib.wbg_tc_wait_limit(ctypes.c_ulonglong(1_000_000)), "wbg_tc_wait_limit")  # 1 ms
        _lib.check(lib.wbg_tc_wait_probe(ctypes.c_void_p(res.data_ptr()),
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "probe")
        torch.cuda.synchronize()
    finally:
        _lib.check(lib.wbg_tc_wait_limit(ctypes.c_ulonglong(DEFAULT_NS)), "wbg_tc_wait_limit")
    assert int(res.item()) == 0  # the wait gave up
    assert _flags() & 1  # WBG_DEVICE_FLAG_TC_TIMEOUT, and cleared again
    assert _flags() == 0


def test_rotation_timeout_then_recovery():
    lib = _lib.load()
    U32, X32, U64, X64 = _rotation_case()
    nk, nF, nw = X32.shape[0], X32.shape[1], 32
    sel, herm = list(range(nF)), [0] * nF
    ref, _ = engine.rotate(U64, X64, nF, sel, herm, nw, nk, True)
    ref = ref.clone()
    _flags()
    try:
        _lib.check(lib.wbg_tc_wait_limit(ctypes.c_ulonglong(0)), "wbg_tc_wait_limit")
        engine.rotate(U32, X32, nF, sel, herm, nw, nk, False)
        torch.cuda.synchronize()
        _flags()  # whether a block gave up depends on timing; the recovery below must hold either way
    finally:
        _lib.check(lib.wbg_tc_wait_limit(ctypes.c_ulonglong(DEFAULT_NS)), "wbg_tc_wait_limit")
    got, _ = engine.rotate(U32, X32, nF, sel, herm, nw, nk, False)
    torch.cuda.synchronize()
    assert _flags() == 0
    err = float((got.to(torch.complex128) - ref).abs().max() / ref.abs().max())
    assert err < 2e-6, err


def test_kubo_timeout_then_recovery():
    """The tensor-core Kubo sums (kubo_tc) with a 0 ns bound on every wait: blocks that find a
    barrier not yet complete give up (producers, issuing thread and epilogue alike), drain their
    products and free their tensor memory; afterwards, with the normal bound, the same run gives
    the same bits as before the timeout and no flag."""
    import wbgpu
    from wbgpu import models, system as wsys
    lib = _lib.load()
    s = wsys.System_R.from_dict(models.config_system(2, small=True))
    s.do_ws_dist(3)
    mk = lambda: {'opt': wbgpu.calculators.OpticalConductivity(Efermi=np.linspace(-0.6, 0.6, 5),
                                                               omega=np.linspace(0.0, 3.0, 200),
                                                               smr_fixed_width=0.1)}
    grid = wbgpu.Grid(s, NKdiv=1, NKFFT=(4, 4, 4))
    before = wbgpu.run(s, grid, mk(), precision='mixed')['opt'].data
    _flags()
    try:
        _lib.check(lib.wbg_tc_wait_limit(ctypes.c_ulonglong(0)), "wbg_tc_wait_limit")
        wbgpu.run(s, grid, mk(), precision='mixed')
        torch.cuda.synchronize()
        _flags()  # whether a block gave up depends on timing; the recovery below must hold either way
    finally:
        _lib.check(lib.wbg_tc_wait_limit(ctypes.c_ulonglong(DEFAULT_NS)), "wbg_tc_wait_limit")
    after = wbgpu.run(s, grid, mk(), precision='mixed')['opt'].data
    torch.cuda.synchronize()
    assert _flags() == 0
    assert np.array_equal(before, after)
