"""GPU tests of the refined eigensolver (wbg_eigh_batched mode | WBG_EIGH_REFINE): the FP32 solve
followed by one Ogita-Aishima step against the double-float / FP64 H, with Rayleigh-Ritz inside
clusters of close eigenvalues.  Replaces np.linalg.eigh of data_K/data_K.py:211-218 like the other
modes: energies against LAPACK to FP64 accuracy, eigenvectors (complex64) no worse than the
double-float solve's (mode | WBG_EIGH_PRECISE_VECTORS), gauge-invariant projectors against LAPACK."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from wbgpu import engine  # noqa: E402

REFINE, PRECISE, LOWER = engine.EIGH_REFINE, engine.EIGH_PRECISE_VECTORS, engine.EIGH_LOWER


def _df64_complex(H):
    return torch.from_numpy(engine._df64_pairs(H)).contiguous().view(torch.complex128).reshape(H.shape)


def _batch(nw, nk, seed, scale=1.0):
    """Random Hermitian matrices; every 5th with planted exact, 1e-9 and 1e-4 splittings and
    eigenvalues rounded to 0.1 (clusters of a few)."""
    rng = np.random.default_rng(seed)
    H = rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw))
    H = scale * (H + H.conj().swapaxes(1, 2))
    for k in range(0, nk, 5):
        w, v = np.linalg.eigh(H[k])
        w[: nw // 2] = np.round(w[: nw // 2] / scale, 1) * scale
        if nw > 2:
            w[1] = w[0] + 1e-9 * scale
        if nw > 6:
            w[5] = w[4] + 1e-4 * scale
        w = np.sort(w)
        H[k] = (v * w) @ v.conj().T
    return 0.5 * (H + H.conj().swapaxes(1, 2))


def _errors(H, E, U):
    """(max energy error, max |U^H U - I|, max residual |U^H H U - E|, max projector error over
    groups of LAPACK eigenvalues closer than 1e-6)."""
    Eref, Vref = np.linalg.eigh(H)
    nw = H.shape[1]
    Uh = U.conj().swapaxes(1, 2)
    orth = np.abs(Uh @ U - np.eye(nw)).max()
    res = np.abs(Uh @ H @ U - E[:, None, :] * np.eye(nw)).max()
    perr = 0.0
    for k in range(H.shape[0]):
        i = 0
        while i < nw:
            j = i + 1
            while j < nw and Eref[k, j] - Eref[k, j - 1] < 1e-6:
                j += 1
            P0 = Vref[k, :, i:j] @ Vref[k, :, i:j].conj().T
            P1 = U[k, :, i:j] @ U[k, :, i:j].conj().T
            perr = max(perr, np.abs(P0 - P1).max())
            i = j
    return np.abs(E - Eref).max(), orth, res, perr


def _run(H, mode, df64_input, flag_expected=0):
    nk, nw = H.shape[:2]
    Ht = (_df64_complex(H) if df64_input else torch.from_numpy(H)).cuda()
    E, U, flag = engine.eigh(Ht, nw * nw, nw, nk, mode=mode)
    torch.cuda.synchronize()
    assert int(flag.item()) == flag_expected
    return E.cpu().numpy(), U.cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("base", [2, 3])
@pytest.mark.parametrize("nw", [1, 2, 5, 8, 17, 32])
def test_refine_vs_lapack(nw, base):
    """Energies within 1e-12 |E| nw of LAPACK (as the FP64 modes); orthonormality, residual and
    projectors of the complex64 vectors within 1.5x (plus a floor of a few FP32 ulps) of the
    double-float solve with precise vectors on the same matrices."""
    H = _batch(nw, 300, 40 + nw)
    Er, Ur = _run(H, base | REFINE, base == 3)
    Ep, Up = _run(H, base | PRECISE, base == 3)
    scale = max(np.abs(Er).max(), 1.0)
    er, orth_r, res_r, perr_r = _errors(H, Er, Ur)
    ep, orth_p, res_p, perr_p = _errors(H, Ep, Up)
    assert er < 1e-12 * scale * nw, (er, ep)
    assert orth_r < 1.5 * orth_p + 4e-7, (orth_r, orth_p)
    assert res_r < 1.5 * res_p + 4e-7 * scale, (res_r, res_p)
    assert perr_r < 1.5 * perr_p + 4e-7, (perr_r, perr_p)


@pytest.mark.parametrize("scale", [1e-3, 30.0])
def test_refine_scales(scale):
    """Small and large spectra (the cluster threshold follows max |lambda|): energies to 1e-12
    relative, projectors to complex64 accuracy."""
    H = _batch(32, 200, 7, scale)
    E, U = _run(H, 3 | REFINE, True)
    e, orth, res, perr = _errors(H, E, U)
    assert e < 1e-12 * np.abs(E).max() * 32
    assert orth < 1e-6 and perr < 2e-6


def test_refine_wide_cluster():
    """A 12-fold degenerate eigenvalue (wider than the 8-column Rayleigh-Ritz block): re-diagonalised
    8 at a time, exact for an exact degeneracy, and reported in errflag (4)."""
    rng = np.random.default_rng(11)
    nw, nk = 32, 40
    H = np.empty((nk, nw, nw), np.complex128)
    for k in range(nk):
        w = np.sort(rng.uniform(-8, 8, nw))
        w[10:22] = 0.7
        w = np.sort(w)
        q = np.linalg.qr(rng.standard_normal((nw, nw)) + 1j * rng.standard_normal((nw, nw)))[0]
        H[k] = (q * w) @ q.conj().T
    H = 0.5 * (H + H.conj().swapaxes(1, 2))
    E, U = _run(H, 3 | REFINE, True, flag_expected=4)
    e, orth, res, perr = _errors(H, E, U)
    assert e < 1e-12 * 8 * nw and orth < 1e-6 and perr < 2e-6, (e, orth, perr)


def test_refine_lower_and_stages():
    """The lower-triangle input gives the same bits as the full matrix; the two-stage split
    (STAGE1, then STAGE2 reading H again) the same bits as one call."""
    nw, nk = 32, 150
    H = _batch(nw, nk, 3)
    Hl = H.copy()
    iu = np.triu_indices(nw, 1)
    Hl[:, iu[0], iu[1]] = np.nan
    E0, U0 = _run(H, 3 | REFINE, True)
    E1, U1 = _run(Hl, 3 | REFINE | LOWER, True)
    assert np.array_equal(E0, E1) and np.array_equal(U0, U1)
    Ht = _df64_complex(H).cuda()
    E2, U2, f = engine.eigh(Ht, nw * nw, nw, nk, mode=3 | REFINE | engine.EIGH_STAGE1)
    E2, U2, f = engine.eigh(Ht, nw * nw, nw, nk, E=E2, U=U2, mode=3 | REFINE | engine.EIGH_STAGE2)
    torch.cuda.synchronize()
    assert np.array_equal(E2.cpu().numpy(), E0) and np.array_equal(U2.cpu().numpy().astype(np.complex128), U0)


@pytest.mark.parametrize("mode", [1 | REFINE, 0 | REFINE, 2 | REFINE | engine.EIGH_VALUES, 2 | REFINE | PRECISE])
def test_refine_bad_modes(mode):
    """The refinement is for modes 2 / 3 with eigenvectors only."""
    H = torch.from_numpy(_batch(8, 4, 1)).cuda()
    with pytest.raises(ValueError):
        engine.eigh(H, 64, 8, 4, mode=mode)


def test_refine_too_large():
    H = torch.zeros((2, 33, 33), dtype=torch.complex128, device='cuda')
    with pytest.raises(ValueError):
        engine.eigh(H, 33 * 33, 33, 2, mode=2 | REFINE)
