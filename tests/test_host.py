"""CPU-only checks: the C-ABI library loads and exports every symbol include/wbgpu.h declares,
and the host-side logic (R-vector structure, phase tables, grids, MDRS) matches the oracle."""
import os
import re

import numpy as np
import pytest

from oracle import wb_oracle as O
from wbgpu import models, engine, system as wsys, grid as wgrid, _lib


REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(REPO, 'include', 'wbgpu.h')).read()
    return sorted(set(re.findall(r'^\s*(?:int|const char\*|size_t)\s+(wbg_\w+)\s*\(', src, re.M)))


def test_header_matches_binding():
    assert header_functions() == sorted(_lib.EXPORTS)


def test_library_loads_and_exports():
    lib = _lib.load()
    for name in header_functions():
        assert hasattr(lib, name), name
    assert lib.wbg_abi_version() == 1
    assert lib.wbg_status_string(5).decode() == "workspace too small"


def test_workspace_queries_without_gpu():
    import ctypes
    lib = _lib.load()
    g = _lib.R2KGeom(nR=10, nw=4, nw2=16, nBase=4, nP=5, nU=3, N0=4, N1=4, N2=4, nk=64, nr0=3, nr1=3, nr2=3,
                     rmin0=-1, rmin1=-1, rmin2=-1, maxPairLen=3, maxSliceLen=3)
    b = ctypes.c_size_t(0)
    assert lib.wbg_r2k_workspace_size(ctypes.byref(g), 1, 2, 1, ctypes.byref(b)) == 0
    assert b.value > 0
    assert lib.wbg_r2k_workspace_size(ctypes.byref(g), 0, 2, 1, ctypes.byref(b)) == 1
    assert lib.wbg_eigh_workspace_size(200, 10, ctypes.byref(b)) == 1
    with pytest.raises(ValueError):
        _lib.check(1, "x")
    with pytest.raises(RuntimeError):
        _lib.check(3, "x")
    assert lib.wbg_last_cuda_error_string().decode()  # "none", or the runtime's message


def test_eigh_flag_words():
    """The eigensolver's error word: bit 0 (QL did not converge) raises, bit 2 (refined solve: a
    cluster wider than the Rayleigh-Ritz block, or a matrix that did not settle) warns."""
    import warnings
    torch = pytest.importorskip("torch")
    engine.check_flags([torch.zeros(1, dtype=torch.int32)])
    with pytest.raises(RuntimeError):
        engine.check_flags([torch.zeros(1, dtype=torch.int32), torch.tensor([1], dtype=torch.int32)])
    with pytest.raises(RuntimeError):
        engine.check_flags([torch.tensor([5], dtype=torch.int32)])
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        engine.check_flags([torch.tensor([4], dtype=torch.int32), torch.zeros(1, dtype=torch.int32)])
    assert any(issubclass(x.category, RuntimeWarning) for x in w)


def test_mixed_eigensolver_plan():
    """The mixed path refines an FP32 solve at 24 < nw <= 32 and keeps the double-float solve with
    precise eigenvectors elsewhere (the mode bits of wbg_eigh_batched); its Berry-curvature dipole
    runs in double-float arithmetic on the complex64 fields."""
    assert engine.EIGH_REFINE == 256 and engine.EIGH_PRECISE_VECTORS == 64
    lo, hi = engine.MIXED_EIGH_REFINE_NW
    assert (lo, hi) == (24, 32) and engine.MIXED_EIGH_REFINE
    assert engine.MIXED_DEROMEGA_ARITH == 2


def test_rgeometry_structure():
    rng = np.random.default_rng(3)
    R = np.unique(rng.integers(-3, 4, size=(80, 3)), axis=0)
    rng.shuffle(R)
    g = engine.RGeometry(R)
    Rs = R[g.order]
    # pairs and slices partition the sorted list exactly
    for p in range(g.nP):
        blk = Rs[g.pair_start[p]:g.pair_start[p + 1]]
        assert np.all(blk[:, :2] == blk[0, :2]) and blk[0, 1] == g.pair_r1[p]
        assert np.all(np.diff(blk[:, 2]) > 0)
    for u in range(g.nU):
        for p in range(g.slice_start[u], g.slice_start[u + 1]):
            assert Rs[g.pair_start[p], 0] == g.slice_r0[u]
    assert g.pair_start[-1] == len(R) and g.slice_start[-1] == g.nP


def test_separable_phases_reproduce_dft():
    """The per-axis tables multiply to exp(2 pi i R.(j/N + dK)), the kernel of fft.py:175-180 with expdK."""
    d = models.config_system(2, small=True)
    g = engine.RGeometry(d['iRvec'])
    N = (3, 4, 5)
    dK = np.array([[0.1, -0.2, 0.3]]) / N
    ph = g.phases(dK, N)
    X = d['XX_R']['Ham'][g.order]
    data = O.DataK(O.RSystem(d['real_lattice'], d['iRvec'], d['wannier_centers_cart'], d['XX_R']), N, dK[0])
    ref = data.R_to_k(data.get_R_mat('Ham'), 0, hermitian=False)
    Rs = g.R - g.rmin
    out = np.zeros_like(ref)
    for ik, (j0, j1, j2) in enumerate(np.ndindex(*N)):
        e = ph[0][0, j0, Rs[:, 0]] * ph[1][0, j1, Rs[:, 1]] * ph[2][0, j2, Rs[:, 2]]
        out[ik] = np.einsum('r,rmn->mn', e, X)
    assert np.max(np.abs(out - ref)) < 1e-12 * np.max(np.abs(ref))


def test_grid_block_shifts_match_reference_layout():
    g = wgrid.Grid(NKdiv=(2, 3, 1), NKFFT=(4, 4, 6))
    assert np.allclose(g.block_shifts(), O.block_shifts((2, 3, 1), (4, 4, 6)))
    assert g.nblocks == 6 and g.nk_per_block == 96


def test_mdrs_matches_oracle():
    d = models.config_system(2, small=True)
    s = wsys.System_R.from_dict(d).do_ws_dist(3)
    o = O.do_ws_dist(O.RSystem(d['real_lattice'], d['iRvec'], d['wannier_centers_cart'], d['XX_R']), (3, 3, 3))
    idx = {tuple(R): i for i, R in enumerate(s.iRvec)}
    assert len(idx) == len(o.iRvec)
    perm = np.array([idx[tuple(R)] for R in o.iRvec])
    for k in o.XX_R:
        assert np.max(np.abs(s._XX_R[k][perm] - o.XX_R[k])) == 0.0


def test_set_R_mat_hermitian_and_errors():
    d = models.config_system(1, small=True)
    s = wsys.System_R(real_lattice=d['real_lattice'], iRvec=d['iRvec'], wannier_centers_cart=None, num_wann=4)
    X = np.random.default_rng(0).standard_normal((s.nRvec, 4, 4)) + 0j
    s.set_R_mat('Ham', X, Hermitian=True)
    H = s.get_R_mat('Ham')
    assert np.allclose(H, s.conj_XX_R(H))
    with pytest.raises(RuntimeError):
        s.set_R_mat('Ham', X)
    with pytest.raises(ValueError):
        s.get_R_mat('AA')


def test_rspace_field_weights_match_reference_derivative():
    """The R-space weights that wbg_r2k_fields applies (i(R + t_n - t_m), curl) are the
    reference's derivative / rotAA (fourier/rvectors.py:487-494, data_K/data_K_R.py:48-51):
    transforming weighted fields reproduces Xbar before rotation."""
    d = models.config_system(2, small=True)
    o = O.RSystem(d['real_lattice'], d['iRvec'], d['wannier_centers_cart'], d['XX_R'])
    data = O.DataK(o, (2, 3, 2), np.array([0.1, 0.2, 0.3]) / 4)
    # host restatement of the kernel's weights for DER1 and ROT
    cR = o.cRvec_shifted()                                   # (nR, nw, nw, 3)
    A = data.get_R_mat('AA')
    rot = 1j * (cR[..., [1, 2, 0]] * A[..., [2, 0, 1]] - cR[..., [2, 0, 1]] * A[..., [1, 2, 0]])
    assert np.allclose(rot, data.get_R_mat('rotAA'))
    dH = 1j * cR * data.get_R_mat('Ham')[..., None]
    assert np.allclose(dH, data.derivative(data.get_R_mat('Ham')))


def test_field_plan_layout():
    desc, index = engine.field_plan({'V', 'A', 'O'}, True, ['AA'])
    assert index == {'H': 0, 'V': 1, 'A': 4, 'O': 7}
    assert desc[0] == (0, 0, 0, 0) and desc[1] == (1, 0, 0, 0) and desc[7] == (3, 1, 0, 0)
    assert engine.order_for({'V', 'A', 'O'}) == 1 and engine.order_for({'W'}) == 2


def test_host_caches_follow_the_matrices():
    """The pinned upload copies and Hermiticity verdicts kept with a system are dropped when
    set_R_mat replaces or adds to a matrix, and all of them when do_ws_dist changes the R-vectors."""
    d = models.config_system(2, small=True)
    s = wsys.System_R.from_dict(d)
    order = np.arange(s.nRvec)
    first = engine.host_pinned(s, 'Ham', order).clone()
    engine.host_pinned(s, 'AA', order)
    s.__dict__.setdefault('_herm_cache', {})[('Ham', 1e-12)] = True
    s.set_R_mat('Ham', 2 * s.get_R_mat('Ham'), reset=True)
    assert ('Ham', 1e-12) not in s._herm_cache and 'AA' in s._pinned_cache
    again = engine.host_pinned(s, 'Ham', order)
    assert np.allclose(again.numpy(), 2 * first.numpy())
    s.do_ws_dist(3)
    assert not s._pinned_cache and not s._herm_cache
    assert engine.host_pinned(s, 'Ham', np.arange(s.nRvec)).shape[1] == s.nRvec


def test_spin_field_plan_and_hermitian_flags():
    """Spin quantities: 9-component keys take 9 bases, SS follows its Hermiticity verdict, SA etc.
    never count as Hermitian."""
    keys = engine.extra_keys_for({'V', 'A', 'S', 'SA', 'SHA'})
    assert keys == ['AA', 'SS', 'SA', 'SHA']
    desc, index = engine.field_plan({'V', 'A', 'S', 'SA', 'SHA'}, False, keys)
    assert [index[q] for q in ('V', 'A', 'S', 'SA', 'SHA')] == [0, 3, 6, 9, 18]
    assert desc[9] == (0, 1 + 3 + 3, 0, 0) and desc[26] == (0, 1 + 3 + 3 + 9 + 8, 0, 0)
    herm = engine.hermitian_fields({'V', 'A', 'S', 'SA'}, False, herm_bases=('Ham', 'AA', 'SS'))
    assert herm == [True] * 9 + [False] * 9
    herm = engine.hermitian_fields({'S'}, False, herm_bases=('Ham', 'AA'))
    assert herm == [False] * 3


def test_reference_static_calculator_names():
    """Every static calculator of the reference (calculators/static.py, test variants aside) is
    reachable by name; those without a GPU kernel raise NotImplementedError when constructed."""
    from wbgpu import calculators as C
    names = ['DOS', 'CumDOS', 'Spin', 'Morb', 'GME_orb_FermiSurf', 'GME_orb_FermiSea', 'GME_spin_FermiSea',
             'GME_spin_FermiSurf', 'AHC', 'Ohmic_FermiSea', 'Ohmic_FermiSurf', 'Hall_classic_FermiSurf',
             'Hall_classic_FermiSea', 'BerryDipole_FermiSurf', 'NLAHC_FermiSurf', 'BerryDipole_FermiSea',
             'NLAHC_FermiSea', 'NLDrude_FermiSea', 'NLDrude_FermiSurf', 'NLDrude_Fermider2', 'eMChA_FermiSurf',
             'NLDrude_Zeeman_spin', 'NLDrude_Zeeman_orb_Omega', 'NLDrude_Zeeman_orb', 'AHC_Zeeman_spin',
             'OmegaOmega', 'AHC_Zeeman_orb', 'SHC', 'QuantumMetric_FermiSea', 'QuantumMetric_Vel_DQ']
    for n in names:
        assert hasattr(C.static, n), n
    for n in C._NO_KERNEL:
        with pytest.raises(NotImplementedError):
            getattr(C.static, n)(Efermi=np.linspace(-1, 1, 5))
    C.static.AHC(Efermi=np.linspace(-1, 1, 5))  # a calculator with a kernel constructs on the CPU


def test_tabulate_and_sdct_names_point_elsewhere():
    from wbgpu import calculators as C
    for ns, names in ((C.tabulate, ['TabulatorAll', 'Energy', 'Velocity', 'BerryCurvature', 'OrbitalMoment']),
                      (C.sdct, ['SDCT_asym', 'SDCT_sym', 'SDCT_sym_sea_I', 'SDCT_asym_surf_II'])):
        for n in names:
            with pytest.raises(NotImplementedError):
                getattr(ns, n)()
    with pytest.raises(NotImplementedError, match=r"wbgpu\.tabulate\(system, grid"):
        C.TabulatorAll({})


def test_deromega_rejects_unknown_arithmetic():
    """wbg_berry_deromega takes fp64 = 0 (FP32), 1 (FP64) or 2 (complex64 fields, double-float
    arithmetic); anything else is a bad argument, refused before any device work."""
    import ctypes
    lib = _lib.load()
    sc = _lib.Scan(EFmin=-1.0, EFmax=1.0, dEF=0.1, degen_thresh=1e-4, nEF=21)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the argument checks come first
    for bad in (3, -1):
        st = lib.wbg_berry_deromega(dummy, dummy, 21, 0, 3, 6, 9, 12, 3, 8, 10, ctypes.byref(sc), 1, 1, dummy,
                                    bad, None)
        assert st == 1, (bad, st)

