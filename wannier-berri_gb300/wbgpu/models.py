"""Seeded synthetic tight-binding models used by the benchmark and the tests.

The workloads are random tight-binding models built from plain arrays (no file
ingestion).  Each generator returns a dict with ``real_lattice`` (3x3, rows are
lattice vectors in Angstrom), ``iRvec`` (nR, 3) integers, ``wannier_centers_cart``
(nw, 3) and ``XX_R`` {key: complex128 array (nR, nw, nw[, 3])}, the same layout
as ``System_R._XX_R`` in the reference (system/system_R.py:83,106-175).

Hermiticity X(-R) = X(R)^dagger is imposed here exactly the way
``System_R.set_R_mat(..., Hermitian=True)`` does it (system/system_R.py:165-166,
fourier/rvectors.py:397-430), so feeding the arrays to either implementation
gives the same input.
"""
import numpy as np


def cube_R(half):
    r = np.arange(-half, half + 1)
    g = np.stack(np.meshgrid(r, r, r, indexing='ij'), axis=-1).reshape(-1, 3)
    return g


def conj_R(iRvec, X):
    """X(R) -> X(-R)^dagger (requires a -R partner for every R)."""
    index = {tuple(R): i for i, R in enumerate(iRvec)}
    minus = np.array([index[tuple(-R)] for R in iRvec])
    return X[minus].swapaxes(1, 2).conj()


def hermitize(iRvec, X):
    return 0.5 * (X + conj_R(iRvec, X))


def _cnormal(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def triclinic_lattice(rng, lengths=(3.0, 5.0), angles=(80.0, 100.0)):
    a, b, c = rng.uniform(*lengths, size=3)
    al, be, ga = np.radians(rng.uniform(*angles, size=3))
    v1 = np.array([a, 0, 0])
    v2 = np.array([b * np.cos(ga), b * np.sin(ga), 0])
    cx = c * np.cos(be)
    cy = c * (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
    cz = np.sqrt(max(c * c - cx * cx - cy * cy, 1e-6))
    v3 = np.array([cx, cy, cz])
    return np.array([v1, v2, v3])


def random_tb(num_wann, half_R, real_lattice, decay_length=1.0, seed=0, centers='zero',
              keys=('Ham', 'AA'), soc_pairs=False):
    """Random TB model: X_R ~ CN(0,1) exp(-|R|/decay_length), Hermitian in R.

    ``Ham`` is in eV with a real onsite diagonal U[-1,1]; ``AA`` (and ``CC``) are
    Hermitian position-like matrices scaled by 0.1 with a real diagonal at R=0;
    ``BB`` is generated like ``AA`` but not symmetrised (it is not Hermitian in
    the reference either).  With ``soc_pairs`` the orbitals are spin-interlaced
    pairs: spin-diagonal hoppings plus Hermitian spin-orbit blocks of ~0.05 eV.
    """
    rng = np.random.default_rng(seed)
    iRvec = cube_R(half_R)
    nR = len(iRvec)
    cR = iRvec.dot(real_lattice)
    decay = np.exp(-np.linalg.norm(cR, axis=1) / decay_length)
    iR0 = int(np.where(np.all(iRvec == 0, axis=1))[0][0])
    nw = num_wann
    if centers == 'zero':
        wcc = np.zeros((nw, 3))
    else:
        wcc_red = rng.uniform(0, 1, size=(nw, 3))
        wcc = wcc_red.dot(real_lattice)
    XX = {}
    if soc_pairs:
        norb = nw // 2
        h = _cnormal(rng, (nR, norb, norb)) * decay[:, None, None]
        H = np.zeros((nR, nw, nw), dtype=complex)
        H[:, 0::2, 0::2] = h
        H[:, 1::2, 1::2] = h
        soc = 0.05 * _cnormal(rng, (nR, norb, norb)) * decay[:, None, None]
        H[:, 0::2, 1::2] += soc
        H[:, 1::2, 0::2] += -soc.conj()
        if centers != 'zero':
            wcc[1::2] = wcc[0::2]
    else:
        H = _cnormal(rng, (nR, nw, nw)) * decay[:, None, None]
    H = hermitize(iRvec, H)
    H[iR0] -= np.diag(np.diag(H[iR0]))
    H[iR0] += np.diag(rng.uniform(-1, 1, size=nw))
    XX['Ham'] = H
    for key in keys:
        if key == 'Ham':
            continue
        X = 0.1 * _cnormal(rng, (nR, nw, nw, 3)) * decay[:, None, None, None]
        if key in ('AA', 'CC'):
            X = hermitize(iRvec, X)
            d = np.arange(nw)
            X[iR0, d, d, :] = X[iR0, d, d, :].real
        XX[key] = X
    return dict(real_lattice=np.array(real_lattice, dtype=float), iRvec=iRvec,
                wannier_centers_cart=wcc, XX_R=XX)


def config_system(config, seed_index=0, small=False):
    """Models of the benchmark configurations, seed = 1000*config + seed_index.

    config 1: cubic a=1, nw=8, R in [-2,2]^3, Ham + AA (AHC at 501 E_F).
    config 2: triclinic (3-5 A, 80-100 deg), nw=32, R in [-4,4]^3, decay 1.5 A,
              random centres; MDRS (mp_grid 9) is applied by the caller.
    config 3: nw=96 spin-interlaced with SOC blocks, R in [-5,5]^3.
    ``small`` shrinks nw / R for fast CPU parity checks of the same structure.
    """
    seed = 1000 * config + seed_index
    rng = np.random.default_rng(seed + 7)
    if config == 1:
        return random_tb(4 if small else 8, 1 if small else 2, np.eye(3), 1.0, seed,
                         keys=('Ham', 'AA'))
    if config == 2:
        lat = triclinic_lattice(rng)
        return random_tb(6 if small else 32, 1 if small else 4, lat, 1.5, seed, centers='random',
                         keys=('Ham', 'AA', 'BB', 'CC'))
    if config == 3:
        lat = triclinic_lattice(rng)
        return random_tb(8 if small else 96, 1 if small else 5, lat, 1.0, seed, centers='random',
                         keys=('Ham', 'AA'), soc_pairs=True)
    raise ValueError(f"unknown config {config}")
