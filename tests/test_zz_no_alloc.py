"""GPU test of wbg_eigh_batched_noalloc, the eigensolver entry point that allocates nothing.

It serves callers that cannot allocate device memory (inside stream capture, under a host
framework that owns the device allocator, or in allocation-free loops): its workspace is a
fixed device array inside libwbgpu.so.  Its results must equal those of the allocating
entry point wbg_eigh_batched on the same input, on consecutive calls that reuse the shared
scratch.  This file is collected last so a failure here does not hide the other tests.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from wbgpu import _lib, engine  # noqa: E402

SCRATCH_BYTES = 32 << 20


def _hermitian_batch(seed, nk, nw):
    rng = np.random.default_rng(seed)
    H = rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw))
    return torch.from_numpy(H + H.conj().swapaxes(1, 2)).cuda()


def _noalloc(lib, H, nw, nk, fp64_vectors):
    E = torch.empty((nk, nw), dtype=torch.float64, device='cuda')
    U = torch.empty((nk, nw, nw), dtype=torch.complex128 if fp64_vectors else torch.complex64, device='cuda')
    flag = torch.zeros(1, dtype=torch.int32, device='cuda')
    st = lib.wbg_eigh_batched_noalloc(ctypes.c_void_p(H.data_ptr()), nw * nw, nw, nk, ctypes.c_void_p(E.data_ptr()),
                                      ctypes.c_void_p(U.data_ptr()), nw * nw, int(fp64_vectors),
                                      ctypes.c_void_p(flag.data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st, E, U, flag


@pytest.mark.parametrize("nw,fp64_vectors", [(32, True), (32, False), (7, True)])
def test_noalloc_matches_allocating_eigh(nw, fp64_vectors):
    lib = _lib.load()
    nk = 1500 if nw == 32 else 4000
    assert nk * (16 * nw * nw + 32 * nw) + 1024 <= SCRATCH_BYTES
    for call in range(2):  # two calls in a row share (and overwrite) the scratch
        H = _hermitian_batch(100 * nw + call, nk, nw)
        E_ref, U_ref, flag_ref = engine.eigh(H, nw * nw, nw, nk, mode=int(fp64_vectors))
        st, E, U, flag = _noalloc(lib, H, nw, nk, fp64_vectors)
        assert st == 0, lib.wbg_status_string(st).decode()
        torch.cuda.synchronize()
        assert int(flag.item()) == 0 and int(flag_ref.item()) == 0
        E, E_ref = E.cpu().numpy(), E_ref.cpu().numpy()
        scale = np.abs(E_ref).max()
        assert np.max(np.abs(E - E_ref)) <= 1e-12 * scale * nw
        # eigenvectors compared through the gauge-invariant projectors |u><u|
        U, U_ref = U.cpu().numpy().astype(np.complex128), U_ref.cpu().numpy().astype(np.complex128)
        tol = 1e-10 if fp64_vectors else 2e-5
        P = np.einsum('kmi,kni->kimn', U[:, :, :4], U[:, :, :4].conj())
        P_ref = np.einsum('kmi,kni->kimn', U_ref[:, :, :4], U_ref[:, :, :4].conj())
        assert np.max(np.abs(P - P_ref)) < tol


def test_noalloc_rejects_oversized_batch():
    lib = _lib.load()
    nw, nk = 32, 4000  # needs ~70 MB of scratch, above the 32 MiB array
    H = torch.zeros((1, nw, nw), dtype=torch.complex128, device='cuda')
    dummy = torch.zeros(1, dtype=torch.int32, device='cuda')
    p = ctypes.c_void_p(H.data_ptr())
    st = lib.wbg_eigh_batched_noalloc(p, 0, nw, nk, p, p, 0, 1, ctypes.c_void_p(dummy.data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 2  # WBG_STATUS_TOO_LARGE, rejected on the host before any launch
