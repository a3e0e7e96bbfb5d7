"""GPU parity: every stage through the C ABI against the CPU oracle (tolerances in each test).

FP64 path: energies to 1e-10 eV, k-space fields to 1e-12 relative, AHC to 1e-9 relative.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import wb_oracle as O  # noqa: E402
from wbgpu import models, engine, system as wsys  # noqa: E402
import wbgpu  # noqa: E402


def osys(d):
    return O.RSystem(d['real_lattice'], d['iRvec'], d['wannier_centers_cart'], d['XX_R'])


def maxrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def c2small():
    d = models.config_system(2, small=True)
    s = wsys.System_R.from_dict(d)
    s.do_ws_dist(3)
    o = O.RSystem(s.real_lattice, s.iRvec, s.wannier_centers_cart, s._XX_R)
    return s, o


@pytest.mark.parametrize("fp64,tol", [(True, 1e-12), (False, 2e-6), (engine.PREC_FP32S, 2e-6)])
@pytest.mark.parametrize("NKFFT", [(4, 3, 5), (2, 2, 2)])
def test_r2k_fields(c2small, fp64, tol, NKFFT):
    s, o = c2small
    dev = engine.DeviceSystem(s)
    dKs = np.array([[0.13, -0.21, 0.37], [0.0, 0.0, 0.0]]) / np.array(NKFFT)
    q = {'V', 'A', 'O', 'W', 'dA', 'dO', 'B', 'C'}
    fields, index, nF, _ = engine.r2k(dev, dKs, NKFFT, q, True, fp64)
    f = fields.cpu().numpy()
    nk = int(np.prod(NKFFT))
    for ib, dK in enumerate(dKs):
        data = O.DataK(o, NKFFT, dK)
        fb = f[ib * nk:(ib + 1) * nk]
        checks = {'H': data.R_to_k(data.get_R_mat('Ham'), 0, hermitian=False)[..., None],
                  'V': data.R_to_k(data.get_R_mat('Ham'), 1, hermitian=False),
                  'W': data.R_to_k(data.get_R_mat('Ham'), 2, hermitian=False).reshape(nk, s.num_wann, s.num_wann, 9),
                  'A': data.R_to_k(data.get_R_mat('AA'), 0, hermitian=False),
                  'dA': data.R_to_k(data.get_R_mat('AA'), 1, hermitian=False).reshape(nk, s.num_wann, s.num_wann, 9),
                  'O': data.R_to_k(data.get_R_mat('rotAA'), 0, hermitian=False),
                  'dO': data.R_to_k(data.get_R_mat('rotAA'), 1, hermitian=False).reshape(nk, s.num_wann, s.num_wann, 9),
                  'B': data.R_to_k(data.get_R_mat('BB'), 0, hermitian=False),
                  'C': data.R_to_k(data.get_R_mat('CC'), 0, hermitian=False)}
        for name, ref in checks.items():
            n = ref.shape[-1]
            got = np.moveaxis(fb[:, index[name]:index[name] + n], 1, -1)
            assert maxrel(got, ref) < tol, (name, ib, maxrel(got, ref))


def test_r2k_double_float_hamiltonian(c2small):
    """H(k) from the double-float transform (48-bit significand) against the oracle's FP64 FFT."""
    s, o = c2small
    dev = engine.DeviceSystem(s)
    NKFFT = (4, 3, 5)
    dK = np.array([[0.13, -0.21, 0.37]]) / np.array(NKFFT)
    fields, index, nF, _ = engine.r2k(dev, dK, NKFFT, set(), True, engine.PREC_DF64)
    raw = fields.cpu().numpy().view(np.float32).reshape(fields.shape[0], nF, s.num_wann, s.num_wann, 4)
    got = (raw[..., 0].astype(np.float64) + raw[..., 1]) + 1j * (raw[..., 2].astype(np.float64) + raw[..., 3])
    data = O.DataK(o, NKFFT, dK[0])
    ref = data.R_to_k(data.get_R_mat('Ham'), 0, hermitian=False)
    assert maxrel(got[:, 0], ref) < 1e-13


@pytest.mark.parametrize("prec", [engine.PREC_FP32, engine.PREC_FP64, engine.PREC_DF64, engine.PREC_FP32S])
def test_r2k_columns_lower_triangle(c2small, prec):
    """wbg_r2k_columns on the lower triangle of the Hermitian fields: those elements are
    bit-identical to the full transform, the others (upper triangles) are left unwritten."""
    s, _ = c2small
    dev = engine.DeviceSystem(s)
    NKFFT = (4, 3, 5)
    dKs = np.array([[0.13, -0.21, 0.37], [0.3, 0.1, -0.2]]) / np.array(NKFFT)
    q = {'V', 'A', 'O', 'B', 'C'}
    full, index, nF, _ = engine.r2k(dev, dKs, NKFFT, q, True, prec)
    full = full.clone()
    out = torch.empty_like(full)
    out.view(torch.float32).fill_(float('nan'))  # both parts (a complex fill leaves imag at 0)
    low, _, _, _ = engine.r2k(dev, dKs, NKFFT, q, True, prec, out=out, lower=True)
    cols, lower = engine.column_list(dev, q, True, True)
    nw = s.num_wann
    a = full.view(torch.int32).reshape(full.shape[0], nF * nw * nw, -1).cpu().numpy()  # raw bits
    b = low.view(torch.int32).reshape(full.shape[0], nF * nw * nw, -1).cpu().numpy()
    c = cols.cpu().numpy()
    assert np.array_equal(a[:, c], b[:, c])
    rest = np.setdiff1d(np.arange(nF * nw * nw), c)
    assert np.isnan(low.view(torch.float32).reshape(b.shape).cpu().numpy()[:, rest]).all()
    # the non-Hermitian B, C fields are complete, the Hermitian ones lower-triangular
    assert [lower[index[k]] for k in ('H', 'V', 'A', 'O', 'B', 'C')] == [True] * 4 + [False] * 2
    assert len(c) == (nF - 6) * nw * (nw + 1) // 2 + 6 * nw * nw


def _df64_complex(H):
    """complex128 numpy -> torch complex128-sized double-float layout (re.hi, re.lo, im.hi, im.lo)."""
    return torch.from_numpy(engine._df64_pairs(H)).contiguous().view(torch.complex128).reshape(H.shape)


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
@pytest.mark.parametrize("nw", [5, 32, 48])
def test_eigh_lower_triangle_input(nw, mode):
    """mode | WBG_EIGH_LOWER reads only the lower triangle: NaN above the diagonal and a
    non-zero imaginary diagonal change nothing against the full Hermitian input."""
    rng = np.random.default_rng(100 + nw)
    nk = 200
    H = rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw))
    H = H + H.conj().swapaxes(1, 2)
    Hl = H.copy()
    iu = np.triu_indices(nw, 1)
    Hl[:, iu[0], iu[1]] = np.nan
    Hl[:, np.arange(nw), np.arange(nw)] += 3.0j
    conv = _df64_complex if mode == 3 else torch.from_numpy
    E0, U0, f0 = engine.eigh(conv(H).cuda(), nw * nw, nw, nk, mode=mode)
    E0, U0 = E0.clone(), U0.clone()
    E1, U1, f1 = engine.eigh(conv(Hl).cuda(), nw * nw, nw, nk, mode=mode | engine.EIGH_LOWER)
    torch.cuda.synchronize()
    assert int(f0.item()) == 0 and int(f1.item()) == 0
    assert torch.equal(E0, E1) and torch.equal(U0, U1)


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("nw", [6, 32])
def test_rotate_lower_triangle_input(fp64, nw):
    """herm | 4: the field is read from its lower triangle (mirrored, real diagonal) -- equal
    to rotating the full Hermitian matrix, for plain, Hermitian-part and diagonal outputs."""
    rng = np.random.default_rng(7 + nw)
    nk = 64
    cdt = torch.complex128 if fp64 else torch.complex64
    X = rng.standard_normal((nk, 3, nw, nw)) + 1j * rng.standard_normal((nk, 3, nw, nw))
    X = X + X.conj().swapaxes(-1, -2)
    U = np.linalg.qr(rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw)))[0]
    Xl = X.copy()
    iu = np.triu_indices(nw, 1)
    Xl[..., iu[0], iu[1]] = np.nan
    Ut = torch.from_numpy(U).to(cdt).cuda()
    Xt = torch.from_numpy(X).to(cdt).cuda()
    Xlt = torch.from_numpy(Xl).to(cdt).cuda()
    sel = [0, 1, 2]
    a, _ = engine.rotate(Ut, Xt, 3, sel, [0, 1, 2], nw, nk, fp64)
    a = a.clone()
    b, _ = engine.rotate(Ut, Xlt, 3, sel, [4, 5, 6], nw, nk, fp64)
    torch.cuda.synchronize()
    assert torch.equal(a[:, :2], b[:, :2])
    d = torch.arange(nw, device=a.device)
    assert torch.equal(a[:, 2, d, d].real, b[:, 2, d, d].real)


@pytest.mark.parametrize("engine_id", [1, 3])
@pytest.mark.parametrize("nF", [1, 4, 9])
@pytest.mark.parametrize("lower", [False, True])
def test_rotate_tensor_core_vs_fp64(nF, lower, engine_id):
    """FP32 rotation at nw = 32 (tcgen05, 3xTF32 products, FP32 accumulation) against the FP64
    CUDA-core rotation: every output mode, field counts that leave partial 128-row tiles, a
    batch that is not a multiple of the persistent grid; the warp-specialised kernel (engine 1)
    and the one-tile-at-a-time kernel (engine 3, the default).  Relative error < 2e-6 of max |Xbar|."""
    from wbgpu import autotune
    autotune.set_value(autotune.ROTATE_ENGINE, 32, 0, engine_id)
    try:
        _rotate_tc_case(nF, lower)
    finally:
        autotune.set_value(autotune.ROTATE_ENGINE, 32, 0, 0)


def _rotate_tc_case(nF, lower):
    nw, nk = 32, 1000
    rng = np.random.default_rng(31 + nF)
    X = rng.standard_normal((nk, nF, nw, nw)) + 1j * rng.standard_normal((nk, nF, nw, nw))
    if lower:
        X = X + X.conj().swapaxes(-1, -2)
    U = np.linalg.qr(rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw)))[0]
    modes = [(f % 3) | (4 if lower else 0) for f in range(nF)]
    sel = list(range(nF))[::-1]
    Xd, Ud = torch.from_numpy(X).cuda(), torch.from_numpy(U).cuda()
    ref, _ = engine.rotate(Ud, Xd, nF, sel, [m & 3 for m in modes], nw, nk, True)
    ref = ref.clone()
    Xl = Xd.to(torch.complex64)
    if lower:  # the upper triangle is not read
        iu = torch.triu_indices(nw, nw, 1)
        Xl[:, :, iu[0], iu[1]] = complex(float('nan'), float('nan'))
    got, _ = engine.rotate(Ud.to(torch.complex64), Xl, nF, sel, modes, nw, nk, False)
    torch.cuda.synchronize()
    assert engine.device_flags() == 0
    got = got.to(torch.complex128)
    d = torch.arange(nw, device=ref.device)
    # the diagonal-only fields (mode 2) are written on their diagonal alone: the scale comes from
    # the written entries
    scale = max(float((ref[:, f, d, d] if m & 3 == 2 else ref[:, f]).abs().max()) for f, m in enumerate(modes))
    for f, m in enumerate(modes):
        if m & 3 == 2:  # diagonal of the Hermitian part only
            err = float((got[:, f, d, d].real - ref[:, f, d, d].real).abs().max())
        else:
            err = float((got[:, f] - ref[:, f]).abs().max())
        assert err < 2e-6 * scale, (f, m, err / scale)


@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("nw", [72, 96, 128])
def test_rotate_large_nw(fp64, nw):
    """Row-panel rotation (nw > 64) against numpy: plain, Hermitian part, diagonal only, and a
    lower-triangle input; FP64 to 1e-12, FP32 to 2e-6 of max |Xbar|."""
    rng = np.random.default_rng(nw)
    nk, nF = 6, 4
    X = rng.standard_normal((nk, nF, nw, nw)) + 1j * rng.standard_normal((nk, nF, nw, nw))
    X[:, 3] = X[:, 3] + X[:, 3].conj().swapaxes(-1, -2)
    U = np.linalg.qr(rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw)))[0]
    U = np.ascontiguousarray(U)
    cdt = torch.complex128 if fp64 else torch.complex64
    Xl = X.copy()
    iu = np.triu_indices(nw, 1)
    Xl[:, 3][:, iu[0], iu[1]] = np.nan
    got, _ = engine.rotate(torch.from_numpy(U).to(cdt).cuda(), torch.from_numpy(Xl).to(cdt).cuda(), nF,
                           [0, 1, 2, 3], [0, 1, 2, 5], nw, nk, fp64)
    got = got.cpu().numpy().astype(np.complex128)
    Y = U.conj().swapaxes(-1, -2)[:, None] @ X @ U[:, None]
    H = 0.5 * (Y + Y.conj().swapaxes(-1, -2))
    tol = (1e-12 if fp64 else 2e-6) * np.abs(Y).max()
    d = np.arange(nw)
    assert np.abs(got[:, 0] - Y[:, 0]).max() < tol
    assert np.abs(got[:, 1] - H[:, 1]).max() < tol
    assert np.abs(got[:, 2][:, d, d].real - H[:, 2][:, d, d].real).max() < tol
    assert np.abs(got[:, 3] - H[:, 3]).max() < tol


@pytest.mark.parametrize("mode", [1, 0, 2])
@pytest.mark.parametrize("nw", [1, 2, 5, 8, 17, 32, 48, 96, 128])
def test_eigh_random(nw, mode):
    """mode 1: FP64; mode 0: FP64 solve + FP32 vectors; mode 2: double-float solve + FP32 vectors.
    Energies to 1e-12 |E| nw in every mode; vectors to FP64 or FP32 accuracy."""
    rng = np.random.default_rng(nw)
    nk = 300
    H = rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw))
    H = H + H.conj().swapaxes(1, 2)
    # planted degeneracies / near-degeneracies in part of the batch
    for k in range(0, nk, 7):
        w, v = np.linalg.eigh(H[k])
        w[: nw // 2] = np.round(w[: nw // 2], 1)
        if nw > 2:
            w[1] = w[0] + 1e-9
        H[k] = (v * w) @ v.conj().T
    Ht = torch.from_numpy(H).cuda()
    E, U, flag = engine.eigh(Ht, nw * nw, nw, nk, mode=mode)
    torch.cuda.synchronize()
    assert int(flag.item()) == 0
    E, U = E.cpu().numpy(), U.cpu().numpy().astype(np.complex128)
    vtol = 1e-10 if mode == 1 else 1e-5
    Href = 0.5 * (H + H.conj().swapaxes(1, 2))
    Eref = np.linalg.eigvalsh(Href)
    scale = np.abs(Eref).max()
    assert np.max(np.abs(E - Eref)) < 1e-12 * max(scale, 1) * nw
    I = np.eye(nw)
    Uh = U.conj().swapaxes(1, 2)
    assert np.max(np.abs(Uh @ U - I)) < vtol
    R = Uh @ Href @ U - E[:, None, :] * I
    assert np.max(np.abs(R)) < 0.1 * vtol * max(scale, 1) * nw


def test_ahc_golden_random(golden_dir):
    """The reference's own golden AHC (tests/reference/integrate_files/random-ahc_iter-0000.npz)."""
    import os
    f = np.load(os.path.join(golden_dir, 'random_system.npz'))
    XX = {k[5:]: f[k] for k in f.files if k.startswith('XX_R_')}
    s = wsys.System_R.from_arrays(f['real_lattice'], f['iRvec'], f['wannier_centers_cart'], XX)
    ref = np.load(os.path.join(golden_dir, 'random_results.npz'))
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=3), {'ahc': wbgpu.calculators.AHC(Efermi=np.linspace(-2, 2, 5))})
    got, exp = res['ahc'].data, ref['ahc_data']
    assert np.max(np.abs(got - exp)) < 1e-8 * np.max(np.abs(exp))


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-9), ('mixed', 1e-6)])
def test_ahc_c1(precision, tol):
    d = models.config_system(1)
    EF = np.linspace(-2, 2, 501)
    s = wsys.System_R.from_dict(d)
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=8), {'ahc': wbgpu.calculators.AHC(Efermi=EF)}, precision=precision)
    ref = O.run(osys(d), (2, 2, 2), (8, 8, 8), {'ahc': O.AHC(Efermi=EF)})
    assert maxrel(res['ahc'].data, ref['ahc'].data) < tol


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-9), ('mixed', 1e-6)])
def test_ahc_c2small_mdrs(c2small, precision, tol):
    s, o = c2small
    EF = np.linspace(-2, 2, 201)
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=(4, 5, 3)), {'ahc': wbgpu.calculators.AHC(Efermi=EF)},
                    precision=precision)
    ref = O.run(o, (2, 2, 2), (4, 5, 3), {'ahc': O.AHC(Efermi=EF)})
    assert maxrel(res['ahc'].data, ref['ahc'].data) < tol


def test_ahc_internal_only(c2small):
    s, o = c2small
    EF = np.linspace(-2, 2, 51)
    kw = dict(kwargs_formula={'external_terms': False})
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=1, NKFFT=4), {'ahc': wbgpu.calculators.AHC(Efermi=EF, **kw)})
    ref = O.run(o, (1, 1, 1), (4, 4, 4), {'ahc': O.AHC(Efermi=EF, **kw)})
    assert maxrel(res['ahc'].data, ref['ahc'].data) < 1e-9


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-9), ('mixed', 1e-6)])
def test_morb_c2small(c2small, precision, tol):
    s, o = c2small
    EF = np.linspace(-2, 2, 101)
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=(3, 4, 3)), {'morb': wbgpu.calculators.Morb(Efermi=EF)},
                    precision=precision)
    ref = O.run(o, (2, 2, 2), (3, 4, 3), {'morb': O.Morb(Efermi=EF)})
    assert maxrel(res['morb'].data, ref['morb'].data) < tol


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-9), ('mixed', 1e-6)])
def test_bcd_c2small(c2small, precision, tol):
    s, o = c2small
    EF = np.linspace(-2, 2, 101)
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=(3, 4, 3)),
                    {'bcd': wbgpu.calculators.BerryDipole_FermiSea(Efermi=EF)}, precision=precision)
    ref = O.run(o, (2, 2, 2), (3, 4, 3), {'bcd': O.BerryDipole_FermiSea(Efermi=EF)})
    assert res['bcd'].data.shape == ref['bcd'].data.shape
    assert maxrel(res['bcd'].data, ref['bcd'].data) < tol


def test_bcd_internal_only(c2small):
    s, o = c2small
    EF = np.linspace(-2, 2, 41)
    kw = dict(kwargs_formula={'external_terms': False})
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=1, NKFFT=4), {'bcd': wbgpu.calculators.BerryDipole_FermiSea(Efermi=EF, **kw)})
    ref = O.run(o, (1, 1, 1), (4, 4, 4), {'bcd': O.BerryDipole_FermiSea(Efermi=EF, **kw)})
    assert maxrel(res['bcd'].data, ref['bcd'].data) < 1e-9


@pytest.mark.parametrize("smr,kBT", [('Lorentzian', 0.0), ('Gaussian', 0.0), ('Lorentzian', 0.05)])
def test_optcond_c3small(smr, kBT):
    d = models.config_system(3, small=True)
    s = wsys.System_R.from_dict(d)
    EF = np.linspace(-1, 1, 11)
    om = np.linspace(0, 4, 40)
    kw = dict(Efermi=EF, omega=om, smr_fixed_width=0.05, smr_type=smr, kBT=kBT)
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=4), {'opt': wbgpu.calculators.OpticalConductivity(**kw)})
    ref = O.run(osys(d), (2, 2, 2), (4, 4, 4), {'opt': O.OpticalConductivity(**kw)})
    # FP64 pair records and band sums (the FP64 path)
    assert maxrel(res['opt'].data, ref['opt'].data) < 1e-9


def test_golden_random_morb_and_opt(golden_dir):
    """The reference's golden random-Morb and random-opt_conductivity (tests/test_run.py:653-669)."""
    import os
    f = np.load(os.path.join(golden_dir, 'random_system.npz'))
    XX = {k[5:]: f[k] for k in f.files if k.startswith('XX_R_')}
    s = wsys.System_R.from_arrays(f['real_lattice'], f['iRvec'], f['wannier_centers_cart'], XX)
    ref = np.load(os.path.join(golden_dir, 'random_results.npz'))
    calcs = {'Morb': wbgpu.calculators.Morb(Efermi=np.linspace(-2, 2, 5)),
             'opt': wbgpu.calculators.OpticalConductivity(Efermi=np.array([17.0, 18.0]), omega=np.arange(0.0, 7.1, 1.0),
                                                         smr_fixed_width=0.20, smr_type="Gaussian")}
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=3), calcs)
    m = ref['Morb_data']
    assert np.max(np.abs(res['Morb'].data - m)) < 1e-8 * np.max(np.abs(m))
    oc = ref['opt_conductivity_data']
    assert np.max(np.abs(res['opt'].data - oc)) < 1e-8 * np.max(np.abs(oc))


def test_ahc_morb_bcd_together(c2small):
    """Calculators sharing one band-data pass: BCD needs the full rotated rotA, AHC/Morb only its diagonal."""
    s, o = c2small
    EF = np.linspace(-2, 2, 61)
    C = wbgpu.calculators
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=4), {'ahc': C.AHC(Efermi=EF), 'morb': C.Morb(Efermi=EF),
                                                        'bcd': C.BerryDipole_FermiSea(Efermi=EF)}, precision='mixed')
    ref = O.run(o, (2, 2, 2), (4, 4, 4), {'ahc': O.AHC(Efermi=EF), 'morb': O.Morb(Efermi=EF),
                                          'bcd': O.BerryDipole_FermiSea(Efermi=EF)})
    for key in ('ahc', 'morb', 'bcd'):
        assert maxrel(res[key].data, ref[key].data) < 1e-6, key


@pytest.fixture(scope="module")
def tb128():
    d = models.random_tb(128, 1, models.triclinic_lattice(np.random.default_rng(3)), 1.5, 4128, centers='random',
                         keys=('Ham', 'AA'))
    return wsys.System_R.from_dict(d)


def test_bcd_large_nw_without_gap_table(tb128):
    """nw = 128, FP64: 2201 Fermi levels leave no room for the per-k 1/(E_x - E_y) table, so the
    kernel recomputes it; every 220th level must equal an 11-level run that uses the table."""
    s = tb128
    grid = wbgpu.Grid(s, NKdiv=1, NKFFT=2)
    ef1, ef2 = np.linspace(-1, 1, 11), np.linspace(-1, 1, 2201)
    r1 = wbgpu.run(s, grid, {'b': wbgpu.calculators.BerryDipole_FermiSea(Efermi=ef1)}, precision='fp64')['b'].data
    r2 = wbgpu.run(s, grid, {'b': wbgpu.calculators.BerryDipole_FermiSea(Efermi=ef2)}, precision='fp64')['b'].data
    assert np.abs(r2[::220] - r1).max() < 1e-10 * np.abs(r1).max()


@pytest.mark.parametrize("nw", [96, 128])
def test_mixed_vs_fp64_large_nw(nw, tb128):
    """Large-nw paths (panel rotation, eigh at n = 96 / 128, Kubo) in mixed precision against FP64."""
    if nw == 128:
        s = tb128
    else:
        d = models.random_tb(96, 1, models.triclinic_lattice(np.random.default_rng(4)), 1.5, 4096, centers='random',
                             keys=('Ham', 'AA'))
        s = wsys.System_R.from_dict(d)
    grid = wbgpu.Grid(s, NKdiv=1, NKFFT=4)
    calcs = lambda: {'ahc': wbgpu.calculators.AHC(Efermi=np.linspace(-1, 1, 21)),
                     'opt': wbgpu.calculators.OpticalConductivity(Efermi=np.linspace(-1, 1, 3),
                                                                  omega=np.linspace(0.1, 2, 16))}
    a = wbgpu.run(s, grid, calcs(), precision='mixed')
    b = wbgpu.run(s, grid, calcs(), precision='fp64')
    # the mixed path's Kubo band sums accumulate in FP32 by design (FP64 energy differences):
    # 1.4e-6 at nw = 128 here, 7e-7 at nw = 96 against the oracle; the Berry curvature to 1e-6
    for key, tol in (('ahc', 1e-6), ('opt', 2e-6)):
        x, y = a[key].data, b[key].data
        assert np.abs(x - y).max() < tol * np.abs(y).max(), (key, np.abs(x - y).max() / np.abs(y).max())


def test_omega_hermitian_column_kernel(c2small):
    """Mixed path: V and A of Xbar are exactly Hermitian, and the column-per-lane Omega kernel
    (wbg_berry_omega fp64 = 2) matches the general FP32 kernel on the same band data (both FP32
    traces; only the summation order differs)."""
    import ctypes
    from wbgpu import _lib
    s, _ = c2small
    dev = engine.DeviceSystem(s)
    NKFFT = (6, 5, 4)
    dKs = np.array([[0.1, 0.2, -0.3], [0.0, 0.5, 0.25]]) / np.array(NKFFT)
    calc = wbgpu.calculators.AHC(Efermi=np.linspace(-2, 2, 41))
    bd = engine.band_data(dev, dKs, NKFFT, calc.quantities(s), 'mixed')
    assert bd.hermitian and bd.omega_mode == 2
    nw = s.num_wann
    iV = bd.index['V']
    V = bd.Xbar[:, iV:iV + 3]
    assert torch.equal(V, V.conj().transpose(-1, -2))
    out = []
    for mode in (2, 0):
        calc.reset(dev.device)
        sc = calc.scan_struct()
        st = _lib.load().wbg_berry_omega(engine._ptr(bd.E), engine._ptr(bd.Xbar), bd.Xbar.shape[1], iV,
                                         bd.index['A'], bd.index['Od'], nw, bd.nk_total, ctypes.byref(sc), 1, 1,
                                         engine._ptr(calc._hist), mode, engine._stream())
        _lib.check(st, "wbg_berry_omega")
        out.append(wbgpu.calculators.fixed_values(calc._hist.cpu().numpy(), calc.nEF_extra * 3))
    assert np.abs(out[0] - out[1]).max() <= 1e-5 * np.abs(out[1]).max()


EVK_QS = ['energy', 'band_gradients', 'berry_curvature', 'berry_curvature_internal_terms',
          'berry_curvature_external_terms']


def _golden_system(golden_dir, name):
    import os
    f = np.load(os.path.join(golden_dir, name))
    XX = {k[5:]: f[k] for k in f.files if k.startswith('XX_R_')}
    return wsys.System_R.from_arrays(f['real_lattice'], f['iRvec'], f['wannier_centers_cart'], XX)


def test_evaluate_k_golden(golden_dir):
    """wbgpu.evaluate_k (FP64) against the reference's own evaluate_k: random system at three
    k-points, Fe (bands 4, 5) at k = (0.1, 0.2, 0.3); rel 1e-8 as tests/test_evaluate_k.py."""
    import os
    g = np.load(os.path.join(golden_dir, 'evaluate_k_ref.npz'))
    rs = _golden_system(golden_dir, 'random_system.npz')
    for i, kp in enumerate(g['random_k']):
        got = wbgpu.evaluate_k(rs, k=kp, quantities=EVK_QS)
        for q in EVK_QS:
            ref = g[f'random_{i}_{q}']
            assert np.allclose(got[q], ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max()), (i, q)
    fe = _golden_system(golden_dir, 'fe_system.npz')
    got = wbgpu.evaluate_k(fe, k=g['fe_k'], quantities=EVK_QS, iband=[4, 5])
    for q in EVK_QS:
        ref = g[f'fe_{q}']
        assert np.allclose(got[q], ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max()), q
    single = wbgpu.evaluate_k(rs, k=g['random_k'][0], quantities=['energy'])
    assert np.allclose(single, g['random_0_energy'], rtol=1e-10)


@pytest.mark.parametrize("precision,tol", [('fp64', 1e-9), ('mixed', 1e-6)])
def test_tabulate_grid_vs_oracle(c2small, precision, tol):
    """Grid tabulation (MDRS system) against the oracle's evaluate_k at every k-point."""
    s, o = c2small
    grid = wbgpu.Grid(s, NKdiv=2, NKFFT=(3, 2, 2))
    tab = wbgpu.tabulate(s, grid, quantities=EVK_QS, precision=precision)
    assert tab['kpoints'].shape == (grid.nblocks * 12, 3)
    for ik in range(0, len(tab['kpoints']), 7):
        ref = O.evaluate_k(o, tab['kpoints'][ik], EVK_QS)
        for q in EVK_QS:
            r = ref[q]
            assert np.abs(tab[q][ik] - r).max() <= tol * max(np.abs(r).max(), 1e-12), (ik, q)


@pytest.mark.parametrize("nw,half,mp", [(6, 1, 3), (16, 2, 5)])
def test_mdrs_device_search_matches_host(nw, half, mp):
    """do_ws_dist with the replica search on the GPU gives exactly the host's replica set and
    matrices (triclinic lattice, random Wannier centres)."""
    d = models.random_tb(nw, half, models.triclinic_lattice(np.random.default_rng(nw)), 1.5, 77 + nw,
                         centers='random', keys=('Ham', 'AA'))
    a = wsys.System_R.from_dict(d).do_ws_dist(mp)
    b = wsys.System_R.from_dict(d).do_ws_dist(mp, device='cuda')
    assert np.array_equal(a.iRvec, b.iRvec)
    for key in ('Ham', 'AA'):
        assert np.array_equal(a.get_R_mat(key), b.get_R_mat(key))


@pytest.mark.parametrize("precision,rule", [('fp64', 1e-8), ('mixed', 1e-6)])
def test_golden_random_dos_ohmic(golden_dir, precision, rule):
    """DOS, CumDOS, Ohmic_FermiSea (inverse mass) and Ohmic_FermiSurf (v v f') against the
    reference's own golden files random-{dos,cumdos,conductivity_ohmic,conductivity_ohmic_fsurf}
    (tests/test_run.py:653-669 settings); FP64 with the reference's 1e-8 rule."""
    import os
    rs = _golden_system(golden_dir, 'random_system.npz')
    ref = np.load(os.path.join(golden_dir, 'random_results.npz'))
    EF = np.linspace(-2, 2, 5)
    C = wbgpu.calculators
    calcs = {'dos': C.DOS(Efermi=EF), 'cumdos': C.CumDOS(Efermi=EF), 'conductivity_ohmic': C.Ohmic_FermiSea(Efermi=EF),
             'conductivity_ohmic_fsurf': C.Ohmic_FermiSurf(Efermi=EF), 'ahc': C.AHC(Efermi=EF)}
    # the reference's random system is not Hermitian in R-space: the mixed path must keep full
    # matrices and the reference's symmetrisation
    assert engine.DeviceSystem(rs).hermitian_bases() == frozenset()
    res = wbgpu.run(rs, wbgpu.Grid(rs, NKdiv=2, NKFFT=3), calcs, precision=precision)
    for key in calcs:
        got, exp = res[key].data, ref[key + '_data']
        assert got.shape == exp.shape, (key, got.shape, exp.shape)
        assert np.abs(got - exp).max() < rule * np.abs(exp).max(), (key, np.abs(got - exp).max() / np.abs(exp).max())


def test_dos_ohmic_c2small_vs_oracle(c2small):
    """Same calculators on the MDRS model against the oracle, FP64 to 1e-9."""
    s, o = c2small
    # the seeded models are Hermitian in R-space: the mixed path takes the lower-triangle route
    assert engine.DeviceSystem(s).hermitian_bases() == frozenset({'Ham', 'AA'})
    EF = np.linspace(-1.5, 1.5, 31)
    C = wbgpu.calculators
    got = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=(4, 3, 3)),
                    {'dos': C.DOS(Efermi=EF), 'cumdos': C.CumDOS(Efermi=EF), 'om': C.Ohmic_FermiSea(Efermi=EF),
                     'os': C.Ohmic_FermiSurf(Efermi=EF)}, precision='fp64')
    ref = O.run(o, (2, 2, 2), (4, 3, 3), {'dos': O.DOS(Efermi=EF), 'cumdos': O.CumDOS(Efermi=EF),
                                          'om': O.Ohmic_FermiSea(Efermi=EF), 'os': O.Ohmic_FermiSurf(Efermi=EF)})
    for key in ('dos', 'cumdos', 'om', 'os'):
        assert maxrel(got[key].data, ref[key].data) < 1e-9, key


# ---------------------------------------------------------------------------------------
# tetrahedron method (tetra=True)
# ---------------------------------------------------------------------------------------
@pytest.mark.parametrize("mode", [1, 3])
@pytest.mark.parametrize("nw", [6, 32])
def test_eigh_values_only(nw, mode):
    """WBG_EIGH_VALUES: the same eigenvalues as the full solve, U untouched (may be NULL)."""
    rng = np.random.default_rng(300 + nw)
    nk = 300
    H = rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw))
    H = H + H.conj().swapaxes(1, 2)
    conv = _df64_complex if mode == 3 else torch.from_numpy
    E0, _, f0 = engine.eigh(conv(H).cuda(), nw * nw, nw, nk, mode=mode)
    E0 = E0.clone()
    E1, U1, f1 = engine.eigh(conv(H).cuda(), nw * nw, nw, nk, mode=mode | engine.EIGH_VALUES)
    torch.cuda.synchronize()
    assert U1 is None and int(f0.item()) == 0 and int(f1.item()) == 0
    assert torch.equal(E0, E1)


def _tetra_calcs(EF, names):
    C = wbgpu.calculators
    cs = {'ahc': C.AHC, 'morb': C.Morb, 'bcd': C.BerryDipole_FermiSea, 'dos': C.DOS, 'cumdos': C.CumDOS,
          'conductivity_ohmic': C.Ohmic_FermiSea, 'conductivity_ohmic_fsurf': C.Ohmic_FermiSurf}
    return {k: cs[k](Efermi=EF, tetra=True) for k in names}


TETRA_ALL = ['ahc', 'morb', 'bcd', 'dos', 'cumdos', 'conductivity_ohmic', 'conductivity_ohmic_fsurf']


@pytest.mark.parametrize("precision,rule", [('fp64', 1e-8), ('mixed', 1e-6)])
def test_tetra_golden_random(golden_dir, precision, rule):
    """All seven static calculators with tetra=True on the reference's random system against
    the reference's own run (tests/golden/tetra_ref.npz); FP64 with the 1e-8 acceptance rule."""
    import os
    rs = _golden_system(golden_dir, 'random_system.npz')
    ref = np.load(os.path.join(golden_dir, 'tetra_ref.npz'))
    res = wbgpu.run(rs, wbgpu.Grid(rs, NKdiv=2, NKFFT=3), _tetra_calcs(ref['EF'], TETRA_ALL), precision=precision)
    for key in TETRA_ALL:
        got, exp = res[key].data, ref['random_' + key]
        assert got.shape == exp.shape, (key, got.shape, exp.shape)
        assert np.abs(got - exp).max() < rule * np.abs(exp).max(), (key, np.abs(got - exp).max() / np.abs(exp).max())


@pytest.mark.parametrize("precision,rule", [('fp64', 1e-9), ('mixed', 1e-6)])
def test_tetra_golden_c2_anisotropic(golden_dir, c2small, precision, rule):
    """Triclinic MDRS model over NKdiv (2,1,3) x NKFFT (3,4,2): every corner lookup of the
    kernels (minus side of block 0 wrapping to the last corner block, index j-1) is exercised."""
    import os
    s, _ = c2small
    ref = np.load(os.path.join(golden_dir, 'tetra_ref.npz'))
    names = ['ahc', 'dos', 'conductivity_ohmic']
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=(2, 1, 3), NKFFT=(3, 4, 2)), _tetra_calcs(ref['EF2'], names),
                    precision=precision)
    for key in names:
        assert maxrel(res[key].data, ref['c2_' + key]) < rule, key


def test_tetra_c1_vs_oracle_blocks():
    """nw = 8 cubic model, a subset of the blocks, 101 levels: GPU vs oracle in FP64; the corner
    energies are computed only for the corner blocks the subset touches."""
    s = wsys.System_R.from_dict(models.config_system(1))
    o = O.RSystem(s.real_lattice, s.iRvec, s.wannier_centers_cart, s._XX_R)
    EF = np.linspace(-2, 2, 101)
    blocks = [0, 5, 7]
    names = ['ahc', 'dos', 'cumdos']
    got = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=(3, 4, 5)), _tetra_calcs(EF, names), precision='fp64',
                    blocks=blocks)
    ocs = {'ahc': O.AHC(Efermi=EF, tetra=True), 'dos': O.DOS(Efermi=EF, tetra=True),
           'cumdos': O.CumDOS(Efermi=EF, tetra=True)}
    ref = O.run(o, (2, 2, 2), (3, 4, 5), ocs, blocks=blocks)
    for key in names:
        assert maxrel(got[key].data, ref[key].data) < 1e-9, key


def test_tetra_cumdos_counts_states():
    """Size-independent property: with E_F above every band CumDOS (tetra) is num_wann states per
    cell, below every band 0; DOS integrates to the same count (trapezoid over a fine grid)."""
    s = wsys.System_R.from_dict(models.config_system(1))
    EF = np.linspace(-12, 12, 2401)
    r = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=6), _tetra_calcs(EF, ['dos', 'cumdos']), precision='mixed')
    cum, dos = r['cumdos'].data, r['dos'].data
    assert abs(cum[0]) < 1e-12 and abs(cum[-1] - s.num_wann) < 1e-9
    assert abs(np.trapezoid(dos, EF) - s.num_wann) < 1e-3 * s.num_wann


def test_tetra_served_equals_run(c2small):
    """tetra=True requests through the Server give run()'s results."""
    s, _ = c2small
    EF = np.linspace(-1.5, 1.5, 31)
    grid = wbgpu.Grid(s, NKdiv=2, NKFFT=3)
    alone = wbgpu.run(s, grid, _tetra_calcs(EF, ['ahc', 'dos']), precision='mixed')
    srv = wbgpu.Server(precision='mixed')
    srv.add_system('c2', s)
    t1 = srv.submit('c2', grid, _tetra_calcs(EF, ['ahc', 'dos']))
    t2 = srv.submit('c2', grid, {'ahc': wbgpu.calculators.AHC(Efermi=EF)})
    srv.run_until_idle()
    r1 = t1.wait()
    t2.wait()
    for key in ('ahc', 'dos'):
        assert maxrel(r1[key].data, alone[key].data) < 1e-9, key


# ---------------------------------------------------------------------------------------
# adaptive refinement (adpt_num_iter)
# ---------------------------------------------------------------------------------------
def test_refine_golden_random(golden_dir):
    """run(adpt_num_iter=3) against the reference's refinement on its random system (FP64, the
    1e-8 rule); the mixed path selects the same K-points and agrees to 1e-6."""
    import os
    from wbgpu.run import run_adaptive
    rs = _golden_system(golden_dir, 'random_system.npz')
    g = np.load(os.path.join(golden_dir, 'refine_ref.npz'))
    C = wbgpu.calculators
    mk = lambda: {'ahc': C.AHC(Efermi=g['EF']), 'dos': C.DOS(Efermi=g['EF']), 'cumdos': C.CumDOS(Efermi=g['EF'])}
    grid = wbgpu.Grid(rs, NKdiv=2, NKFFT=3)
    res = wbgpu.run(rs, grid, mk(), precision='fp64', adpt_num_iter=3, adpt_mesh=2)
    for key in ('ahc', 'dos', 'cumdos'):
        exp = g['random_' + key]
        assert np.abs(res[key].data - exp).max() < 1e-8 * np.abs(exp).max(), key
    dev = engine.DeviceSystem(rs)
    r64, K64, _, f64 = run_adaptive(rs, grid, mk(), 'fp64', dev, 3)
    rm, Km, _, fm = run_adaptive(rs, grid, mk(), 'mixed', dev, 3)
    assert np.array_equal(K64, Km) and np.array_equal(f64, fm)
    for key in ('ahc', 'dos', 'cumdos'):
        assert np.abs(rm[key].data - r64[key].data).max() < 1e-6 * np.abs(r64[key].data).max(), key


def test_refine_golden_c2_anisotropic(golden_dir, c2small):
    """Triclinic MDRS model: adpt_fac 2, adpt_mesh (2, 1, 3), AHC and Berry-curvature dipole."""
    import os
    s, _ = c2small
    g = np.load(os.path.join(golden_dir, 'refine_ref.npz'))
    C = wbgpu.calculators
    res = wbgpu.run(s, wbgpu.Grid(s, NKdiv=2, NKFFT=(3, 4, 2)),
                    {'ahc': C.AHC(Efermi=g['EF2']), 'bcd': C.BerryDipole_FermiSea(Efermi=g['EF2'])},
                    precision='fp64', adpt_num_iter=2, adpt_mesh=(2, 1, 3), adpt_fac=2)
    for key in ('ahc', 'bcd'):
        assert maxrel(res[key].data, g['c2_' + key]) < 1e-9, key


def test_refine_served_equals_run(c2small):
    """A request with refinement rounds through the Server (next to a plain request) gives run()'s
    adaptive result."""
    s, _ = c2small
    EF = np.linspace(-1.5, 1.5, 31)
    C = wbgpu.calculators
    grid = wbgpu.Grid(s, NKdiv=2, NKFFT=3)
    alone = wbgpu.run(s, grid, {'ahc': C.AHC(Efermi=EF)}, precision='mixed', adpt_num_iter=2, adpt_fac=2)
    srv = wbgpu.Server(precision='mixed')
    srv.add_system('c2', s)
    t1 = srv.submit('c2', grid, {'ahc': C.AHC(Efermi=EF)}, adpt_num_iter=2, adpt_fac=2)
    t2 = srv.submit('c2', grid, {'dos': C.DOS(Efermi=EF)})
    srv.run_until_idle()
    r1 = t1.wait()
    t2.wait()
    assert maxrel(r1['ahc'].data, alone['ahc'].data) < 1e-9
    from wbgpu.run import run_adaptive
    _, K, _, _ = run_adaptive(s, grid, {'ahc': C.AHC(Efermi=EF)}, 'mixed', engine.DeviceSystem(s), 2, 2, 2)
    assert t1.nkpoints == len(K) * 27 and len(K) > 8  # every K-point of every round, 3^3 k each


@pytest.mark.parametrize("precision,rule", [('fp64', 1e-8), ('mixed', 1e-6)])
def test_refine_tetra_golden(golden_dir, precision, rule):
    """tetra=True with adaptive refinement against the reference: refined K-points get the 8
    corner grids of their own cell (wbg_tetra_grid.per_block)."""
    import os
    rs = _golden_system(golden_dir, 'random_system.npz')
    g = np.load(os.path.join(golden_dir, 'refine_ref.npz'))
    C = wbgpu.calculators
    res = wbgpu.run(rs, wbgpu.Grid(rs, NKdiv=2, NKFFT=3),
                    {'ahc': C.AHC(Efermi=g['EF'], tetra=True), 'dos': C.DOS(Efermi=g['EF'], tetra=True)},
                    precision=precision, adpt_num_iter=2, adpt_mesh=2)
    for key in ('ahc', 'dos'):
        exp = g['tetra_random_' + key]
        assert np.abs(res[key].data - exp).max() < rule * np.abs(exp).max(), key


def test_refine_tetra_served(c2small):
    """The same through the Server (corner grids per refined block on the request's stream)."""
    s, _ = c2small
    EF = np.linspace(-1.5, 1.5, 31)
    C = wbgpu.calculators
    grid = wbgpu.Grid(s, NKdiv=2, NKFFT=3)
    mk = lambda: {'ahc': C.AHC(Efermi=EF, tetra=True)}
    alone = wbgpu.run(s, grid, mk(), precision='mixed', adpt_num_iter=1)
    srv = wbgpu.Server(precision='mixed')
    srv.add_system('c2', s)
    t = srv.submit('c2', grid, mk(), adpt_num_iter=1)
    srv.run_until_idle()
    assert maxrel(t.wait()['ahc'].data, alone['ahc'].data) < 1e-9
