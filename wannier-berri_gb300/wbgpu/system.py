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
        self._drop_host_caches(key)
        if key in self._XX_R:
            if reset:
                self._XX_R[key] = value
            elif add:
                self._XX_R[key] = self._XX_R[key] + value
            else:
                raise RuntimeError(f"setting {key} for the second time without explicit permission")
        else:
            self._XX_R[key] = value

    def _drop_host_caches(self, key=None):
        """Forget what the engine derived from the matrices on the host (pinned upload copies,
        Hermiticity verdicts): for `key`, or all of them when the R-vectors change."""
        for name in ('_pinned_cache', '_herm_cache'):
            cache = self.__dict__.get(name)
            if cache is None:
                continue
            if key is None:
                cache.clear()
            else:
                for k in [k for k in cache if k == key or (isinstance(k, tuple) and k[0] == key)]:
                    del cache[k]

    @property
    def NKFFT_recommended(self):
        if getattr(self, '_NKFFT_recommended', None) is not None:
            return self._NKFFT_recommended
        rec = np.ones(3, dtype=int)
        for i in range(3):
            R = self.iRvec[:, i]
            rec[i] += max(R.max(), 0) - min(R.min(), 0)
        return rec

    def do_ws_dist(self, mp_grid, ws_dist_tol=1e-5, device=None):
        """MDRS: replace (iRvec, XX_R) by the Wigner-Seitz replica set (system/system_R.py:572-588).
        device: None searches the replicas on the host, 'cuda' with the wbg_ws_replicas kernel."""
        mp = np.array(mp_grid if np.ndim(mp_grid) else [mp_grid] * 3, dtype=int)
        self._drop_host_caches()
        self.iRvec, self._XX_R = mdrs_remap(self.real_lattice, self.wannier_centers_red, self.iRvec,
                                            self._XX_R, mp, ws_dist_tol, device=device)
        self._NKFFT_recommended = mp
        return self


def _grid_points(mp):
    g = np.stack(np.meshgrid(*[np.arange(n) for n in mp], indexing='ij'), axis=-1)
    return g.reshape(-1, 3)


def _ws_search_host(real_lattice, ushift, pts, sup, tol):
    """Replica search on the host: for every shift s and grid point p, the supercell offsets q
    with the smallest |(pts[p] + sup[q] + s) L|, ties within tol -> flat (s, p, q) arrays."""
    cRs = (pts[:, None, :] + sup[None, :, :]).dot(real_lattice)  # (npt, nsup, 3)
    out_s, out_p, out_q = [], [], []
    for si, sh in enumerate(ushift):
        dist = np.linalg.norm(cRs + sh.dot(real_lattice), axis=2)
        sel = np.abs(dist - dist.min(axis=1, keepdims=True)) < tol
        p, q = np.nonzero(sel)
        out_s.append(np.full(len(p), si))
        out_p.append(p)
        out_q.append(q)
    return np.concatenate(out_s), np.concatenate(out_p), np.concatenate(out_q)


def _ws_search_device(real_lattice, ushift, pts, sup, tol, device):
    """The same search with the wbg_ws_replicas kernel (one thread per (shift, grid point))."""
    import ctypes
    import torch
    from . import _lib
    lib = _lib.load()
    dev = torch.device(device)
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)
    sh, pt, su = t(ushift, np.float64), t(pts, np.int32), t(sup, np.int32)
    lat = _lib.Lattice()
    for i, v in enumerate(np.asarray(real_lattice, dtype=float).reshape(-1)):
        lat.L[i] = float(v)
    nS, npt = len(ushift), len(pts)
    maxrep = 8
    while True:
        count = torch.empty((nS, npt), dtype=torch.int32, device=dev)
        repq = torch.empty((nS, npt, maxrep), dtype=torch.int32, device=dev)
        st = lib.wbg_ws_replicas(ctypes.c_void_p(sh.data_ptr()), nS, ctypes.c_void_p(pt.data_ptr()), npt,
                                 ctypes.c_void_p(su.data_ptr()), len(sup), ctypes.byref(lat), ctypes.c_double(tol),
                                 maxrep, ctypes.c_void_p(count.data_ptr()), ctypes.c_void_p(repq.data_ptr()),
                                 ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
        _lib.check(st, "wbg_ws_replicas")
        c = count.cpu().numpy()
        if c.max() <= maxrep:
            break
        maxrep = int(c.max())
    r = repq.cpu().numpy()
    s_idx, p_idx = np.nonzero(np.ones_like(c, dtype=bool))
    n = c.reshape(-1)
    keep = np.arange(maxrep)[None, :] < n[:, None]
    return (np.repeat(s_idx, n), np.repeat(p_idx, n), r.reshape(-1, maxrep)[keep])


def mdrs_remap(real_lattice, wcc_red, iRvec_old, XX_R, mp, tol=1e-5, search=3, device=None):
    """Vectorised MDRS.  For every distinct centre shift t_n - t_m (rounded like
    rvectors.py:75-82) each mp-grid point is mapped to its Wigner-Seitz-nearest
    replicas R (distance ties within ``tol``), the matrix element divided by the
    number of replicas.  All-zero R-vectors are dropped (rvectors.py:111-123).
    ``device``: None searches on the host, a CUDA device runs the search kernel; both give
    the same replica sets."""
    nw = wcc_red.shape[0]
    ndig = int(np.ceil(-np.log10(tol))) + 1
    shifts = np.round(-wcc_red[:, None, :] + wcc_red[None, :, :], ndig).reshape(-1, 3)
    ushift, sidx = np.unique(shifts, axis=0, return_inverse=True)
    sidx = sidx.reshape(-1)
    pts = _grid_points(mp)
    sup = np.stack(np.meshgrid(*[np.arange(-search, search + 1)] * 3, indexing='ij'), axis=-1).reshape(-1, 3) * mp
    if device is None:
        rs, rp, rq = _ws_search_host(real_lattice, ushift, pts, sup, tol)
    else:
        rs, rp, rq = _ws_search_device(real_lattice, ushift, pts, sup, tol, device)
    # replicas sorted by shift: rows start[s] .. start[s+1] belong to shift s
    order = np.lexsort((rq, rp, rs))
    rs, rp, rq = rs[order], rp[order], rq[order]
    ndeg = np.zeros((len(ushift), len(pts)), dtype=np.int64)
    np.add.at(ndeg, (rs, rp), 1)
    rw = 1.0 / ndeg[rs, rp]
    rR = pts[rp] + sup[rq]
    start = np.searchsorted(rs, np.arange(len(ushift) + 1))
    # grid representation of the old matrices: sum of R-vectors equal mod mp
    gidx_old = np.ravel_multi_index(tuple((iRvec_old % mp).T), tuple(mp))
    allR, iR = np.unique(rR, axis=0, return_inverse=True)
    iR = iR.reshape(-1)
    # every (m, n) takes the replicas of its shift: one flat scatter for all elements
    lens = (start[1:] - start[:-1])[sidx]
    mn = np.repeat(np.arange(nw * nw), lens)
    offs = np.arange(lens.sum()) - np.repeat(np.cumsum(lens) - lens, lens)
    ridx = start[sidx[mn]] + offs
    m_e, n_e = np.divmod(mn, nw)
    new = {}
    for key, X in XX_R.items():
        g = np.zeros((len(pts),) + X.shape[1:], dtype=complex)
        np.add.at(g, gidx_old, X)
        out = np.zeros((len(allR),) + X.shape[1:], dtype=complex)
        w = rw[ridx].reshape((-1,) + (1,) * (X.ndim - 3))
        out[iR[ridx], m_e, n_e] = g[rp[ridx], m_e, n_e] * w
        new[key] = out
    keep = np.zeros(len(allR), dtype=bool)
    for X in new.values():
        keep |= np.abs(X.reshape(len(allR), -1)).max(axis=1) > 1e-8
    return allR[keep], {k: v[keep] for k, v in new.items()}
