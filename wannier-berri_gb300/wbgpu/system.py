"""Host-side mirror of the reference ``System_R`` container and its MDRS setup.

``System_R`` here holds what the hot path reads -- lattice, R-vectors, Wannier
centres and the real-space matrices ``_XX_R[key]`` of shape (nR, nw, nw[, 3]) --
with the reference's method names (system/system_R.py:18-212, 572-588).
``do_ws_dist`` builds the MDRS (Wigner-Seitz replica) R-set with 1/N_degen weights
folded into the matrices (fourier/rvectors.py:57-227,570-609); it is a vectorised
host implementation of that setup step (not timed in the benchmark).
"""
import numpy as np


class System_R:
    """Minimal ``System_R``: ``real_lattice`` rows are lattice vectors (Angstrom)."""

    def __init__(self, real_lattice=None, iRvec=None, wannier_centers_cart=None, num_wann=None,
                 force_internal_terms_only=False, periodic=(True, True, True), name='wbgpu'):
        self.real_lattice = None if real_lattice is None else np.array(real_lattice, dtype=float)
        self.iRvec = None if iRvec is None else np.array(iRvec, dtype=int)
        self.num_wann = num_wann
        self.wannier_centers_cart = None if wannier_centers_cart is None else np.array(wannier_centers_cart, float)
        self.force_internal_terms_only = force_internal_terms_only
        self.periodic = np.array(periodic, dtype=bool)
        self.name = name
        self._XX_R = {}

    @classmethod
    def from_arrays(cls, real_lattice, iRvec, wannier_centers_cart, XX_R, **kw):
        s = cls(real_lattice=real_lattice, iRvec=iRvec, wannier_centers_cart=wannier_centers_cart,
                num_wann=XX_R['Ham'].shape[1], **kw)
        for k, v in XX_R.items():
            s.set_R_mat(k, np.array(v, dtype=complex))
        return s

    @classmethod
    def from_dict(cls, d, **kw):
        return cls.from_arrays(d['real_lattice'], d['iRvec'], d['wannier_centers_cart'], d['XX_R'], **kw)

    # --- reference-named accessors (system/system_R.py:106-175, system/system.py:174-181)
    @property
    def nRvec(self):
        return self.iRvec.shape[0]

    @property
    def cell_volume(self):
        return abs(np.linalg.det(self.real_lattice))

    @property
    def wannier_centers_red(self):
        return self.wannier_centers_cart.dot(np.linalg.inv(self.real_lattice))

    @property
    def Ham_R(self):
        return self.get_R_mat('Ham')

    def has_R_mat(self, key):
        return key in self._XX_R

    def get_R_mat(self, key):
        try:
            return self._XX_R[key]
        except KeyError:
            raise ValueError(f"The real-space matrix elements '{key}' are not set in the system,"
                             " but are required for the current calculation.")

    def conj_XX_R(self, XX_R):
        """X(R) -> X(-R)^dagger; R-vectors without a -R partner give zero (rvectors.py:372-430)."""
        index = {tuple(R): i for i, R in enumerate(self.iRvec)}
        out = np.zeros(XX_R.shape, dtype=complex)
        src = np.array([index.get(tuple(-R), -1) for R in self.iRvec])
        ok = src >= 0
        out[ok] = XX_R[src[ok]]
        return out.swapaxes(1, 2).conj()

    def set_R_mat(self, key, value, Hermitian=False, reset=False, add=False):
        value = np.asarray(value)
        if self.num_wann is None:
            self.num_wann = value.shape[1]
        assert value.shape[0] == self.nRvec and value.shape[1:3] == (self.num_wann, self.num_wann), \
            f"{key}: expected shape ({self.nRvec}, {self.num_wann}, {self.num_wann}, ...), got {value.shape}"
        if Hermitian:
            value = 0.5 * (value + self.conj_XX_R(value))
        if key in self._XX_R:
            if reset:
                self._XX_R[key] = value
            elif add:
                self._XX_R[key] = self._XX_R[key] + value
            else:
                raise RuntimeError(f"setting {key} for the second time without explicit permission")
        else:
            self._XX_R[key] = value

    @property
    def NKFFT_recommended(self):
        if getattr(self, '_NKFFT_recommended', None) is not None:
            return self._NKFFT_recommended
        rec = np.ones(3, dtype=int)
        for i in range(3):
            R = self.iRvec[:, i]
            rec[i] += max(R.max(), 0) - min(R.min(), 0)
        return rec

    def do_ws_dist(self, mp_grid, ws_dist_tol=1e-5):
        """MDRS: replace (iRvec, XX_R) by the Wigner-Seitz replica set (system/system_R.py:572-588)."""
        mp = np.array(mp_grid if np.ndim(mp_grid) else [mp_grid] * 3, dtype=int)
        self.iRvec, self._XX_R = mdrs_remap(self.real_lattice, self.wannier_centers_red, self.iRvec,
                                            self._XX_R, mp, ws_dist_tol)
        self._NKFFT_recommended = mp
        return self


def _grid_points(mp):
    g = np.stack(np.meshgrid(*[np.arange(n) for n in mp], indexing='ij'), axis=-1)
    return g.reshape(-1, 3)


def mdrs_remap(real_lattice, wcc_red, iRvec_old, XX_R, mp, tol=1e-5, search=3):
    """Vectorised MDRS.  For every distinct centre shift t_n - t_m (rounded like
    rvectors.py:75-82) each mp-grid point is mapped to its Wigner-Seitz-nearest
    replicas R (distance ties within ``tol``), the matrix element divided by the
    number of replicas.  All-zero R-vectors are dropped (rvectors.py:111-123)."""
    nw = wcc_red.shape[0]
    ndig = int(np.ceil(-np.log10(tol))) + 1
    shifts = np.round(-wcc_red[:, None, :] + wcc_red[None, :, :], ndig).reshape(-1, 3)
    ushift, sidx = np.unique(shifts, axis=0, return_inverse=True)
    sidx = sidx.reshape(nw, nw)
    pts = _grid_points(mp)
    sup = np.stack(np.meshgrid(*[np.arange(-search, search + 1)] * 3, indexing='ij'), axis=-1).reshape(-1, 3) * mp
    iRs = pts[:, None, :] + sup[None, :, :]                 # (npt, nsup, 3)
    cRs = iRs.dot(real_lattice)
    # grid representation of the old matrices: sum of R-vectors equal mod mp
    gidx_old = np.ravel_multi_index(tuple((iRvec_old % mp).T), tuple(mp))
    grids = {}
    for key, X in XX_R.items():
        g = np.zeros((len(pts),) + X.shape[1:], dtype=complex)
        np.add.at(g, gidx_old, X)
        grids[key] = g
    replicas = []
    for s in ushift:
        dist = np.linalg.norm(cRs + s.dot(real_lattice), axis=2)
        sel = np.abs(dist - dist.min(axis=1, keepdims=True)) < tol
        ndeg = sel.sum(axis=1)
        p, q = np.nonzero(sel)
        replicas.append((iRs[p, q], p, 1.0 / ndeg[p]))
    allR = np.unique(np.concatenate([r[0] for r in replicas]), axis=0)
    off = allR.min(axis=0)
    span = allR.max(axis=0) - off + 1
    code = lambda R: np.ravel_multi_index(tuple((R - off).T), tuple(span))
    lookup = np.full(np.prod(span), -1, dtype=np.int64)
    lookup[code(allR)] = np.arange(len(allR))
    new = {key: np.zeros((len(allR),) + g.shape[1:], dtype=complex) for key, g in grids.items()}
    for si, (R, p, w) in enumerate(replicas):
        ms, ns = np.nonzero(sidx == si)
        iR = lookup[code(R)]
        for key, g in grids.items():
            extra = (1,) * (g.ndim - 3)
            new[key][iR[:, None], ms[None, :], ns[None, :]] = \
                g[p[:, None], ms[None, :], ns[None, :]] * w.reshape((-1, 1) + extra)
    keep = np.zeros(len(allR), dtype=bool)
    for X in new.values():
        keep |= np.abs(X.reshape(len(allR), -1)).max(axis=1) > 1e-8
    return allR[keep], {k: v[keep] for k, v in new.items()}
