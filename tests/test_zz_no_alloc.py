"""GPU test of wbg_eigh_batched_noalloc, the eigensolver entry point that allocates nothing.

It serves callers that cannot allocate device memory: a plugin inside an application whose
memory manager owns the GPU's memory, a real-time loop that forbids allocation after start-up
(cudaMalloc may synchronise the device), or an FFI binding without a device allocator.  Its
workspace is a fixed device array inside libwbgpu.so.  Its results must equal those of the
allocating entry point wbg_eigh_batched on the same input, on consecutive calls that reuse
the shared scratch, in every solve precision, with lower-triangle input and for eigenvalues
only.  This file is collected last so a failure here does not hide the other tests.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from wbgpu import _lib, engine  # noqa: E402

SCRATCH_BYTES = 32 << 20
LOWER, VALUES, STAGE1, STAGE2 = 4, 8, 16, 32


def _hermitian_batch(seed, nk, nw, mode):
    """H on the device in the input type of the mode: complex128, or double-float complex
    (hi, lo float pairs per component) for mode 3; with LOWER the upper triangle holds NaN."""
    rng = np.random.default_rng(seed)
    H = rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw))
    H = H + H.conj().swapaxes(1, 2)
    if mode & LOWER:
        iu = np.triu_indices(nw, 1)
        H[:, iu[0], iu[1]] = np.nan
    if (mode & 3) == 3:
        re_hi, im_hi = H.real.astype(np.float32), H.imag.astype(np.float32)
        re_lo = (H.real - re_hi).astype(np.float32)
        im_lo = (H.imag - im_hi).astype(np.float32)
        return torch.from_numpy(np.ascontiguousarray(np.stack([re_hi, re_lo, im_hi, im_lo], -1))).cuda()
    return torch.from_numpy(H).cuda()


def _noalloc(lib, H, nw, nk, mode):
    E = torch.empty((nk, nw), dtype=torch.float64, device='cuda')
    U = None
    if not mode & VALUES:
        U = torch.empty((nk, nw, nw), dtype=torch.complex128 if (mode & 3) == 1 else torch.complex64, device='cuda')
    flag = torch.zeros(1, dtype=torch.int32, device='cuda')
    st = lib.wbg_eigh_batched_noalloc(ctypes.c_void_p(H.data_ptr()), nw * nw, nw, nk, ctypes.c_void_p(E.data_ptr()),
                                      None if U is None else ctypes.c_void_p(U.data_ptr()), nw * nw, int(mode),
                                      ctypes.c_void_p(flag.data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st, E, U, flag


@pytest.mark.parametrize("nw,mode", [(32, 1), (32, 0), (7, 1), (32, 2 | LOWER), (32, 3 | LOWER), (17, 3),
                                     (32, 3 | LOWER | VALUES), (96, 3 | LOWER)])
def test_noalloc_matches_allocating_eigh(nw, mode):
    lib = _lib.load()
    nk = max(1, min(4000, (SCRATCH_BYTES - 1024) // (16 * nw * nw + 32 * nw)) - 100)
    assert nk * (16 * nw * nw + 32 * nw) + 1024 <= SCRATCH_BYTES
    for call in range(2):  # two calls in a row share (and overwrite) the scratch
        H = _hermitian_batch(100 * nw + 10 * mode + call, nk, nw, mode)
        E_ref, U_ref, flag_ref = engine.eigh(H, nw * nw, nw, nk, mode=mode)
        st, E, U, flag = _noalloc(lib, H, nw, nk, mode)
        assert st == 0, lib.wbg_status_string(st).decode()
        torch.cuda.synchronize()
        assert int(flag.item()) == 0 and int(flag_ref.item()) == 0
        E, E_ref = E.cpu().numpy(), E_ref.cpu().numpy()
        scale = np.abs(E_ref).max()
        # the same kernels on the same input: the same energies (to the solver's precision)
        assert np.max(np.abs(E - E_ref)) <= 1e-12 * scale * nw
        if mode & VALUES:
            continue
        # eigenvectors compared through the gauge-invariant projectors |u><u|
        U, U_ref = U.cpu().numpy().astype(np.complex128), U_ref.cpu().numpy().astype(np.complex128)
        tol = 1e-10 if (mode & 3) == 1 else 2e-5
        P = np.einsum('kmi,kni->kimn', U[:, :, :4], U[:, :, :4].conj())
        P_ref = np.einsum('kmi,kni->kimn', U_ref[:, :, :4], U_ref[:, :, :4].conj())
        assert np.max(np.abs(P - P_ref)) < tol


def test_noalloc_rejects_oversized_batch_and_split_stages():
    lib = _lib.load()
    H = torch.zeros((1, 32, 32), dtype=torch.complex128, device='cuda')
    dummy = torch.zeros(1, dtype=torch.int32, device='cuda')
    p = ctypes.c_void_p(H.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    f = ctypes.c_void_p(dummy.data_ptr())
    # nw = 32, nk = 4000 needs ~70 MB of scratch, above the 32 MiB array: rejected on the host
    assert lib.wbg_eigh_batched_noalloc(p, 0, 32, 4000, p, p, 0, 1, f, s) == 2  # WBG_STATUS_TOO_LARGE
    # the two-stage split and a missing U without VALUES are argument errors, nothing launches
    assert lib.wbg_eigh_batched_noalloc(p, 0, 32, 1, p, p, 0, 1 | STAGE1, f, s) == 1
    assert lib.wbg_eigh_batched_noalloc(p, 0, 32, 1, p, p, 0, 1 | STAGE2, f, s) == 1
    assert lib.wbg_eigh_batched_noalloc(p, 0, 32, 1, p, None, 0, 1, f, s) == 1
    torch.cuda.synchronize()
