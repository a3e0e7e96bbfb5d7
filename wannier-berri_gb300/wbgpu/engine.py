"""GPU engine: R-space matrices resident on the device, one pipeline launch per batch of
FFT blocks: R->k fields (wbg_r2k) -> eigh (wbg_eigh_batched) -> U^dagger X U (wbg_rotate).

The band-basis data it produces (``BandData``) is what the reference's ``Data_K``
hands to its formulae (data_K/data_K.py:211-334): E_K, UU_K and the rotated
matrices Xbar(name, der).  Device memory comes from PyTorch; every kernel runs in
libwbgpu.so through the C ABI.  There is no CPU fallback: without a CUDA device or
without the library every entry point raises.
"""
import copy
import ctypes
import warnings

import numpy as np
import torch

from . import _lib

# quantity -> (base kind, r2k kind, components, hermitian after rotation, derivative order)
#   V  = Xbar('Ham', 1)   W = Xbar('Ham', 2)   A = Xbar('AA')    dA = Xbar('AA', 1)
#   O  = Xbar('rotAA')    dO = Xbar('rotAA', 1)   B = Xbar('BB')   C = Xbar('CC')
QUANTITIES = {
    'V': dict(order=1, herm=0, ncomp=3),
    'W': dict(order=2, herm=0, ncomp=9),
    'A': dict(order=0, herm=1, ncomp=3),
    'dA': dict(order=1, herm=1, ncomp=9),
    'O': dict(order=1, herm=1, ncomp=3),
    'Od': dict(order=1, herm=2, ncomp=3),  # rotA when only its diagonal is read (Omega, Morb_Hpm)
    'dO': dict(order=2, herm=1, ncomp=9),
    'B': dict(order=0, herm=0, ncomp=3),
    'C': dict(order=0, herm=0, ncomp=3),
    # spin matrices (system_R.py; SpinVelocity, formula/covariant.py:689-756): S = Xbar('SS')
    # (Hermitian), SH = Xbar('SH'), and the (velocity a, spin s) pairs at 3 a + s of
    # SA, SHA, SR, SHR
    'S': dict(order=0, herm=1, ncomp=3),
    'SH': dict(order=0, herm=0, ncomp=3),
    'SA': dict(order=0, herm=0, ncomp=9),
    'SHA': dict(order=0, herm=0, ncomp=9),
    'SR': dict(order=0, herm=0, ncomp=9),
    'SHR': dict(order=0, herm=0, ncomp=9),
    # dS = Xbar('SS', 1): the derivative of the spin matrices, (spin a, direction d) at 3 a + d
    'dS': dict(order=1, herm=1, ncomp=9),
}
QUANTITY_ORDER = ['V', 'A', 'O', 'Od', 'W', 'dA', 'dO', 'B', 'C', 'S', 'SH', 'SA', 'SHA', 'SR', 'SHR', 'dS']
# R-space key of each plain (moment-0) quantity and the components of every extra key
MOM0_KEY = {'B': 'BB', 'C': 'CC', 'S': 'SS', 'SH': 'SH', 'SA': 'SA', 'SHA': 'SHA', 'SR': 'SR', 'SHR': 'SHR'}
KEY_NCOMP = {'AA': 3, 'BB': 3, 'CC': 3, 'SS': 3, 'SH': 3, 'SA': 9, 'SHA': 9, 'SR': 9, 'SHR': 9}
MOM0, DER1, DER2, ROT, DROT = 0, 1, 2, 3, 4


class StageTimer:
    """CUDA events recorded on the launching (current) stream around each stage call."""

    def __init__(self):
        self.events = {}

    def wrap(self, name, fn, *a, **k):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        r = fn(*a, **k)
        e.record()
        self.events.setdefault(name, []).append((s, e))
        return r

    def totals_ms(self):
        torch.cuda.synchronize()
        return {k: sum(s.elapsed_time(e) for s, e in v) for k, v in self.events.items()}

    def counts(self):
        return {k: len(v) for k, v in self.events.items()}


_TIMER = None
_INDEX_CACHE = {}


def set_timer(timer):
    global _TIMER
    _TIMER = timer


def _timed(name, fn, *a, **k):
    if _TIMER is None:
        return fn(*a, **k)
    return _TIMER.wrap(name, fn, *a, **k)


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("wbgpu needs a CUDA device (sm_103a); no CPU fallback exists")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class RGeometry:
    """Sorted R-vector structure for the pruned separable R->k transform."""

    def __init__(self, iRvec):
        iRvec = np.asarray(iRvec, dtype=np.int64)
        self.order = np.lexsort((iRvec[:, 2], iRvec[:, 1], iRvec[:, 0]))
        R = iRvec[self.order]
        self.R = R
        new_pair = np.ones(len(R), dtype=bool)
        new_pair[1:] = np.any(R[1:, :2] != R[:-1, :2], axis=1)
        self.pair_start = np.append(np.nonzero(new_pair)[0], len(R)).astype(np.int32)
        pairs = R[self.pair_start[:-1]]
        new_slice = np.ones(len(pairs), dtype=bool)
        new_slice[1:] = pairs[1:, 0] != pairs[:-1, 0]
        self.slice_start = np.append(np.nonzero(new_slice)[0], len(pairs)).astype(np.int32)
        self.pair_r1 = pairs[:, 1].astype(np.int32)
        self.slice_r0 = pairs[self.slice_start[:-1], 0].astype(np.int32)
        self.r2 = R[:, 2].astype(np.int32)
        self.rmin = R.min(axis=0)
        self.nr = R.max(axis=0) - self.rmin + 1
        self.nP = len(pairs)
        self.nU = len(self.slice_r0)
        self.maxPairLen = int(np.diff(self.pair_start).max())
        self.maxSliceLen = int(np.diff(self.slice_start).max())

    def phases(self, dKs, NKFFT, step=None):
        """Per-axis tables exp(2 pi i R_d (j s_d + dK_d)) for every block, s_d = 1/N_d (the FFT
        grid of fft.py:179, rvectors.py:467-468) or the per-axis `step` of a sub-grid (a block of
        N_d points spaced by step_d): list of 3 arrays (nblocks, N_d, nr_d) complex128."""
        dKs = np.atleast_2d(dKs)
        out = []
        for d in range(3):
            Rd = self.rmin[d] + np.arange(self.nr[d])
            sd = 1.0 / NKFFT[d] if step is None else float(step[d])
            k = np.arange(NKFFT[d])[None, :] * sd + dKs[:, d][:, None]     # (nb, N)
            out.append(np.exp(2j * np.pi * k[:, :, None] * Rd[None, None, :]))
        return out


def host_pinned(system, key, order):
    """Pinned host copy of XX_R[key] in sorted R order, [ncomp][nR][nw*nw] complex128,
    cached on the system object so repeated uploads start from page-locked memory."""
    cache = system.__dict__.setdefault('_pinned_cache', {})
    if key not in cache:
        X = system.get_R_mat(key)[order]
        nR, nw = X.shape[0], X.shape[1]
        nc = int(np.prod(X.shape[3:]))  # trailing component axes flattened in C order
        a = np.moveaxis(X.reshape(nR, nw * nw, nc), 2, 0)
        t = torch.from_numpy(np.ascontiguousarray(a))
        cache[key] = t.pin_memory() if torch.cuda.is_available() else t
    return cache[key]


class Workspace:
    """Grow-only arena of named device buffers.  Every batch of a run reuses the same buffers
    (stream order makes that safe); concurrent runs on different streams use separate
    workspaces."""

    def __init__(self, device):
        self.device = torch.device(device)
        self._bufs = {}
        # bumped whenever a buffer is (re)allocated: CUDA graphs captured over this workspace's
        # buffers hold their addresses and are valid only while the generation is unchanged
        self.generation = 0
        self.graphs = {}

    def buffer(self, name, shape, dtype):
        """Buffer `name` viewed as dtype[shape], grown when too small (old contents dropped)."""
        nbytes = int(np.prod(shape)) * torch.empty((), dtype=dtype).element_size()
        buf = self._bufs.get(name)
        if buf is None or buf.numel() < nbytes:
            self._bufs.pop(name, None)
            buf = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=self.device)
            self._bufs[name] = buf
            self.generation += 1
        return buf[:nbytes].view(dtype).view(shape)

    def side_stream(self):
        """A second CUDA stream of this workspace (independent stages of one batch)."""
        if getattr(self, '_side', None) is None:
            self._side = torch.cuda.Stream(device=self.device)
        return self._side

    def nbytes(self):
        return sum(b.numel() for b in self._bufs.values())

    def release(self):
        self.graphs.clear()  # graphs first: they hold the buffers' addresses
        self._bufs.clear()
        self.generation += 1


class DeviceSystem:
    """R-space matrices of one system resident on the GPU (uploaded once)."""

    def __init__(self, system, device='cuda'):
        require_cuda()
        _lib.load()
        self.system = system
        self.device = torch.device(device)
        self.nw = system.num_wann
        # the R-vector structure is host metadata of the system: kept with it, keyed by its R-vectors
        iR = np.ascontiguousarray(system.iRvec, dtype=np.int64)
        gkey = (iR.shape, hash(iR.tobytes()))
        cached = system.__dict__.get('_rgeom')
        if cached is None or cached[0] != gkey:
            cached = (gkey, RGeometry(iR))
            system.__dict__['_rgeom'] = cached
        self.geom = cached[1]
        self.lattice = np.array(system.real_lattice, dtype=float)
        self.wcc = np.array(system.wannier_centers_cart, dtype=float)
        self._cache = {}
        self.h2d_bytes = 0

    def hermitian_bases(self, rtol=1e-12):
        """Base matrices whose R-space data are Hermitian, X_R = X_{-R}^dagger within rtol of
        max |X| with every -R present: for them the k-space fields are exactly Hermitian and the
        mixed path transforms only lower triangles.  Other bases keep the full-matrix path with
        the reference's symmetrisation.  The verdict is a property of the host matrices: it is
        computed on the device once and kept with the system's pinned upload copies (dropped
        when set_R_mat or do_ws_dist change the matrices)."""
        if 'herm_bases' not in self._cache:
            verdicts = self.system.__dict__.setdefault('_herm_cache', {})
            out = set()
            for key in ('Ham', 'AA', 'SS'):
                if not self.system.has_R_mat(key):
                    continue
                if (key, rtol) not in verdicts:
                    verdicts[(key, rtol)] = self._hermitian_on_device(key, rtol)
                if verdicts[(key, rtol)]:
                    out.add(key)
            self._cache['herm_bases'] = frozenset(out)
        return self._cache['herm_bases']

    def _hermitian_on_device(self, key, rtol):
        R = self.geom.R  # sorted by (R0, R1, R2): -R found by a binary search on the packed keys
        span = 2 * int(np.abs(R).max()) + 1
        pack = lambda a: ((a[:, 0] * span) + a[:, 1]) * span + a[:, 2]
        keys = pack(R)
        pos = np.minimum(np.searchsorted(keys, pack(-R)), len(keys) - 1)
        if not np.array_equal(keys[pos], pack(-R)):
            return False
        neg = torch.from_numpy(pos).to(self.device)
        nw = self.nw
        X = self._key_fp64(key).reshape(-1, len(R), nw, nw)  # device, sorted R order
        Xd = X[:, neg].conj().transpose(2, 3)
        diff, mx = (X - Xd).abs().max(), X.abs().max()
        return float(diff) <= rtol * max(float(mx), 1e-300)

    def bases_for(self, keys):
        """Base-field list for the R->k launch: Ham, then the components of each extra key."""
        names = [('Ham', None)]
        for key in keys:
            if key != 'Ham':
                names += [(key, c) for c in range(KEY_NCOMP[key])]
        return names

    def _key_fp64(self, key):
        """Device copy (FP64, sorted R order) of one real-space matrix, [ncomp][nR][nw*nw]."""
        ck = ('R', key)
        if ck not in self._cache:
            host = host_pinned(self.system, key, self.geom.order)
            self._cache[ck] = host.to(self.device, non_blocking=True)
            self.h2d_bytes += host.numel() * host.element_size()
        return self._cache[ck]

    def XR(self, names, fp64):
        """Base fields [nBase][nR][nw*nw] for one R->k launch (FP32 copies are cast on the device)."""
        ck = (tuple(names), fp64)
        if ck not in self._cache:
            parts = []
            for key, c in names:
                t = self._key_fp64(key)
                parts.append(t[0:1] if c is None else t[c:c + 1])
            t = torch.cat(parts, dim=0).contiguous()
            self._cache[ck] = t if fp64 else t.to(torch.complex64)
        return self._cache[ck]

    def geom_tensors(self):
        if 'geom' not in self._cache:
            g = self.geom
            mk = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).to(self.device)
            self._cache['geom'] = dict(pair_start=mk(g.pair_start), r2=mk(g.r2), slice_start=mk(g.slice_start),
                                       pair_r1=mk(g.pair_r1), slice_r0=mk(g.slice_r0), iR=mk(g.R))
        return self._cache['geom']

    def buffer(self, name, shape, dtype):
        """Persistent device buffer of the system's default workspace (grow-only), viewed as
        `dtype[shape]`: keeps GB-sized per-batch allocations out of the caching allocator's way."""
        return self.workspace().buffer(name, shape, dtype)

    def workspace(self):
        if 'ws' not in self._cache:
            self._cache['ws'] = Workspace(self.device)
        return self._cache['ws']

    def side_stream(self):
        return self.workspace().side_stream()

    def grid_phases(self, shifts, NKFFT, prec, step=None, cache=True):
        """Device-resident per-axis phase tables for every block of a grid (built once per grid):
        the three tables of one precision go up in one copy (from page-locked memory when large).
        `step`: per-axis spacing of sub-grid blocks (RGeometry.phases).  cache=False: tables of
        blocks used once (refinement sub-grids), not kept by the system: returns (tables, staging
        buffer), the staging buffer to be kept alive until the copy has run."""
        shifts = np.ascontiguousarray(shifts, dtype=np.float64)
        skey = (tuple(int(n) for n in NKFFT), hash(shifts.tobytes()), shifts.shape,
                None if step is None else tuple(float(x) for x in step))
        key = ('phases',) + skey + (int(prec),)
        if not cache:
            return self._upload_phases(self.geom.phases(shifts, NKFFT, step), prec)
        if key not in self._cache:
            hkey = ('phases_host',) + skey
            if hkey not in self._cache:
                self._cache[hkey] = self.geom.phases(shifts, NKFFT, step)
            tabs, host = self._upload_phases(self._cache[hkey], prec)
            self._cache[key] = tabs
            self._cache[key + ('staging',)] = host  # page-locked source of the in-flight copy
        return self._cache[key]

    def _upload_phases(self, tables, prec):
        parts = []
        for p in tables:
            if prec == PREC_DF64:
                parts.append(_df64_pairs(p))
            else:
                parts.append(p.astype(np.complex128 if prec == PREC_FP64 else np.complex64))
        # one flat buffer of the tables' real words (float64 for FP64, float32 otherwise); every
        # table starts on a multiple of its element size
        words = [a.reshape(-1).view(np.float64 if a.dtype == np.complex128 else np.float32) for a in parts]
        host = torch.from_numpy(np.concatenate(words))
        if torch.cuda.is_available() and host.numel() * host.element_size() > (4 << 20):
            host = host.pin_memory()  # large tables: asynchronous copy from page-locked memory
        dev_flat = host.to(self.device, non_blocking=host.is_pinned())
        tabs, off = [], 0
        for a, w in zip(parts, words):
            t = dev_flat[off:off + w.size]
            off += w.size
            if np.iscomplexobj(a):
                t = torch.view_as_complex(t.view(-1, 2))
            tabs.append(t.view(a.shape))
        return tabs, host

    def wcc_tensor(self, fp64):
        k = ('wcc', fp64)
        if k not in self._cache:
            self._cache[k] = torch.tensor(self.wcc, dtype=torch.float64 if fp64 else torch.float32,
                                          device=self.device).contiguous()
        return self._cache[k]


def field_plan(quantities, with_H, extra_keys):
    """Field descriptors (kind, base, a, b) for the requested quantities.
    Bases: 0 = Ham, then the components of each key of ``extra_keys`` in order (AA x/y/z, ...)."""
    base_of = {'Ham': 0}
    nb = 1
    for key in extra_keys:
        base_of[key] = nb
        nb += KEY_NCOMP[key]
    desc, index = [], {}
    if with_H:
        index['H'] = 0
        desc.append((MOM0, 0, 0, 0))
    for q in QUANTITY_ORDER:
        if q not in quantities:
            continue
        index[q] = len(desc)
        if q == 'V':
            desc += [(DER1, 0, a, 0) for a in range(3)]
        elif q == 'W':
            desc += [(DER2, 0, a, b) for a in range(3) for b in range(3)]
        elif q == 'A':
            desc += [(MOM0, base_of['AA'] + b, 0, 0) for b in range(3)]
        elif q == 'dA':
            desc += [(DER1, base_of['AA'] + b, d, 0) for b in range(3) for d in range(3)]
        elif q in ('O', 'Od'):
            desc += [(ROT, base_of['AA'], g, 0) for g in range(3)]
        elif q == 'dO':
            desc += [(DROT, base_of['AA'], g, d) for g in range(3) for d in range(3)]
        elif q == 'dS':
            desc += [(DER1, base_of['SS'] + a, d, 0) for a in range(3) for d in range(3)]
        elif q in MOM0_KEY:
            desc += [(MOM0, base_of[MOM0_KEY[q]] + a, 0, 0) for a in range(QUANTITIES[q]['ncomp'])]
    return desc, index


def hermitian_fields(quantities, with_H, herm_bases=('Ham', 'AA')):
    """Per field of field_plan: True when the k-space field is exactly Hermitian -- its base
    (Ham for H and its derivatives, AA for A, its derivatives and curl, SS for S) is in
    `herm_bases`, the bases whose R-space matrices satisfy X_R = X_{-R}^dagger
    (DeviceSystem.hermitian_bases).  The other keys (BB, CC, SH, SA, SHA, SR, SHR) are never taken
    as Hermitian."""
    keys = extra_keys_for(quantities)
    desc, _ = field_plan(quantities, with_H, keys)
    nonherm = set() if 'Ham' in herm_bases else {0}
    base = 1
    for key in keys:
        if key not in ('AA', 'SS') or key not in herm_bases:
            nonherm |= set(range(base, base + KEY_NCOMP[key]))
        base += KEY_NCOMP[key]
    return [d[1] not in nonherm for d in desc]


def column_list(dev, quantities, with_H, lower):
    """Device int32 list of the elements f*nw2 + m*nw + n that wbg_r2k_columns computes: the
    lower triangle (m >= n) of the Hermitian fields when ``lower``, every element otherwise."""
    key = ('cols', tuple(sorted(quantities)), with_H, bool(lower))
    if key not in dev._cache:
        nw = dev.nw
        herm = hermitian_fields(quantities, with_H, dev.hermitian_bases())
        m, n = np.meshgrid(np.arange(nw), np.arange(nw), indexing='ij')
        full = (m * nw + n).reshape(-1)
        tril = (m * nw + n)[m >= n]
        cols = np.concatenate([f * nw * nw + (tril if (lower and h) else full) for f, h in enumerate(herm)])
        dev._cache[key] = (torch.tensor(cols.astype(np.int32), device=dev.device),
                           [bool(lower and h) for h in herm])
    return dev._cache[key]


def split_columns(dev, quantities, with_H, lower, first):
    """column_list split into (columns of the fields of the quantities in `first`, the rest), for
    a transform that computes two groups of fields in two precisions into one output array."""
    key = ('cols_split', tuple(sorted(quantities)), with_H, bool(lower), tuple(sorted(first)))
    if key not in dev._cache:
        cols, lower_in = column_list(dev, quantities, with_H, lower)
        _, index = field_plan(quantities, with_H, extra_keys_for(quantities))
        nw2 = dev.nw * dev.nw
        f = cols.cpu().numpy() // nw2
        sel = np.zeros(len(lower_in), dtype=bool)
        for q in first:
            if q in index:
                sel[index[q]:index[q] + QUANTITIES[q]['ncomp']] = True
        c = cols.cpu().numpy()
        dev._cache[key] = (torch.tensor(c[sel[f]], device=dev.device), torch.tensor(c[~sel[f]], device=dev.device))
    return dev._cache[key]


def extra_keys_for(quantities):
    keys = []
    if quantities & {'A', 'dA', 'O', 'Od', 'dO'}:
        keys.append('AA')
    for q in QUANTITY_ORDER:
        if q in quantities and q in MOM0_KEY:
            keys.append(MOM0_KEY[q])
    if 'dS' in quantities and 'SS' not in keys:
        keys.append('SS')
    return keys


def order_for(quantities):
    return max([QUANTITIES[q]['order'] for q in quantities] + [0])


class BandData:
    """Band-basis data of a batch of FFT blocks (the reference Data_K content).
    ``index['O']`` (full rotA) also answers diagonal-only requests (``index['Od']``).

    E: (nk_tot, nw) float64; U: (nk_tot, nw, nw) complex128 (view into ``Ubuf``);
    Xbar: (nk_tot, nF, nw, nw) complex (float64 or float32 parts); index: quantity -> first field.
    """

    def __init__(self, E, U, Xbar, index, nblocks, nk, nw, fp64_fields, hermitian=False):
        self.E, self.U, self.Xbar, self.index = E, U, Xbar, index
        self.nblocks, self.nk, self.nw = nblocks, nk, nw
        self.fp64_fields = fp64_fields
        self.hermitian = hermitian  # V and A of Xbar exactly Hermitian (mixed path)
        self.tetra = None  # TetraCorners context, set by run() for tetra=True calculators

    @property
    def omega_mode(self):
        """`fp64` argument of wbg_berry_omega: 1 FP64, 2 FP32 with exactly Hermitian V, A, 0 FP32."""
        return 1 if self.fp64_fields else (2 if self.hermitian else 0)

    @property
    def nk_total(self):
        return self.nblocks * self.nk

    def block(self, b):
        """View of block b alone (per-block results, e.g. for adaptive refinement)."""
        sl = slice(b * self.nk, (b + 1) * self.nk)
        sub = BandData(self.E[sl], None if self.U is None else self.U[sl], None if self.Xbar is None else self.Xbar[sl],
                       self.index, 1, self.nk, self.nw, self.fp64_fields, hermitian=self.hermitian)
        sub._flag = getattr(self, '_flag', None)
        sub._keep = getattr(self, '_keep', None)
        if self.tetra is not None:
            sub.tetra = self.tetra
            sub.tetra_blocks = self.tetra_blocks[b:b + 1]
            sub.tetra_sel = {}
        return sub


def r2k_geometry(dev, NKFFT):
    g = dev.geom
    nw = dev.nw
    return _lib.R2KGeom(nR=len(g.R), nw=nw, nw2=nw * nw, nBase=0, nP=g.nP, nU=g.nU,
                        N0=NKFFT[0], N1=NKFFT[1], N2=NKFFT[2], nk=int(np.prod(NKFFT)),
                        nr0=int(g.nr[0]), nr1=int(g.nr[1]), nr2=int(g.nr[2]),
                        rmin0=int(g.rmin[0]), rmin1=int(g.rmin[1]), rmin2=int(g.rmin[2]),
                        maxPairLen=g.maxPairLen, maxSliceLen=g.maxSliceLen)


PREC_FP32, PREC_FP64, PREC_DF64, PREC_FP32S, PREC_DF64C = 0, 1, 2, 3, 4
# PREC_FP32S: FP32 transform whose k-independent R-space inputs carry a rounding residual
# (hi + lo pair), so they enter with 48 bits; output, intermediates and phases as PREC_FP32.
# PREC_DF64C: double-float transform (inputs, phases and intermediates as PREC_DF64) whose
# output is rounded once to complex64.
C64_PRECS = (PREC_FP32, PREC_FP32S, PREC_DF64C)
DF64_PRECS = (PREC_DF64, PREC_DF64C)


def _input_prec(prec):
    """Precision of the R-space arrays and phase tables a transform of precision `prec` reads."""
    return PREC_DF64 if prec == PREC_DF64C else prec
EIGH_LOWER = 4  # wbg_eigh_batched mode bit: H given by its lower triangle
EIGH_VALUES = 8  # wbg_eigh_batched mode bit: eigenvalues only
EIGH_STAGE1, EIGH_STAGE2 = 16, 32  # wbg_eigh_batched mode bits: tridiagonalise / finish
EIGH_PRECISE_VECTORS = 64  # wbg_eigh_batched mode bit: back-transform in the solve's precision
EIGH_DF64_VECTORS = 128  # with EIGH_PRECISE_VECTORS: U kept in double-float complex
EIGH_REFINE = 256  # wbg_eigh_batched mode bit: FP32 solve + one refinement step against H (nw <= 32)
# Above this num_wann the mixed path rotates in double-float (U, fields and products, Xbar rounded
# to complex64): the FP32 rotation, fields and U errors grow with nw (AHC at nw = 96: 4.5e-6,
# 6.4e-6, 9.5e-6 each against the oracle), the rotation is O(nw^3) and the tensor-core kernel
# serves nw = 32 only.
MIXED_FP32_ROTATION_MAX_NW = 32
# Eigenvectors of the mixed path: back-transformed in double-float and rounded to complex64 once.
# The FP32 back-transform loses ~sqrt(nw) ulps in U, which dominated the mixed path's error
# against the oracle (AHC at nw = 32: 6.6e-7 of the 8.1e-7 total; nw = 96: 9.5e-6).
MIXED_EIGH_BITS = EIGH_PRECISE_VECTORS
# MIXED_EIGH_REFINE_NW[0] < nw <= [1]: the FP32 solve refined against the double-float H
# (EIGH_REFINE) instead: eigenvectors as accurate as the double-float back-transform gives them
# (|U^H U - I| 3.6e-8 against 3.7e-8 on random nw = 32 matrices), energies to ~1e-13 |H|, in 8.5
# instead of 14.0 ms per 55 296 matrices at nw = 32.  The refinement takes a warp per matrix; at
# nw <= 16 the double-float solve packs several matrices per warp and stays faster (the nw = 8
# configuration: 21.8 M k-points/s against 18.1 M refined), and at num_wann 18 and 21 of the
# batched benchmark's systems the refined solve put the Berry-curvature dipole 1.1-1.3e-6 from the
# FP64 path (0.5-0.8e-6 with the double-float solve): the refinement serves 24 < nw <= 32.
MIXED_EIGH_REFINE = True
MIXED_EIGH_REFINE_NW = (24, 32)
# Transform precision of the mixed path's other k-space fields (lower triangles), and the
# quantities whose fields are transformed in double-float (rounded to complex64) whatever it is:
# the velocity, whose FP32 transform error enters D = V / dE (AHC at nw = 32 against the oracle:
# 8.1e-7 with every field in FP32, 2.3e-7 with V in double-float and the precise eigenvectors; the
# Berry-curvature dipole on two 12^3 blocks: 1.9e-6 and 4.8e-7).
MIXED_FIELDS_PREC = 3  # PREC_FP32S
MIXED_DF64_QUANTITIES = {'V'}
# Arithmetic of the mixed path's Berry-curvature dipole (wbg_berry_deromega fp64 argument): 2 =
# double-float on the complex64 band-basis fields.  Its sums over intermediate bands of V D terms
# cancel strongly near degeneracies; in FP32 they put the BCD of a num_wann = 82 system 3.9e-6 from
# the FP64 path (the complex64 rounding of the fields alone: 6e-8).
MIXED_DEROMEGA_ARITH = 2


def _prec(p):
    """precision argument: bool (True = FP64, False = FP32) or PREC_* code"""
    if p is True:
        return PREC_FP64
    if p is False:
        return PREC_FP32
    return int(p)


def _df64_pairs(z):
    """complex128 array -> float32 array [..., 4] = (re.hi, re.lo, im.hi, im.lo) (double-float layout)."""
    parts = []
    for x in (z.real, z.imag):
        hi = x.astype(np.float32)
        lo = (x - hi.astype(np.float64)).astype(np.float32)
        parts += [hi, lo]
    return np.stack(parts, axis=-1)


def _complex_tensor(shape, prec, device):
    """storage for complex values of precision prec (double-float uses complex128-sized slots)"""
    return torch.empty(shape, dtype=torch.complex64 if prec in C64_PRECS else torch.complex128, device=device)


def field_arrays(dev, quantities, with_H, prec):
    """R-space arrays XF[f][R][mn] of the requested k-space fields (wbg_r2k_fields), cached on
    the device system: the derivative / curl weights depend on the system only, not on dK."""
    prec = _input_prec(_prec(prec))
    keys = extra_keys_for(quantities)
    desc, index = field_plan(quantities, with_H, keys)
    ck = ('XF', tuple(sorted(quantities)), with_H, prec)
    if ck not in dev._cache:
        names = dev.bases_for(keys)
        X = dev.XR(names, True)
        nR, nw = len(dev.geom.R), dev.nw
        lat = _lib.Lattice()
        for i, v in enumerate(dev.lattice.reshape(-1)):
            lat.L[i] = float(v)
        fd = torch.tensor(np.array(desc, dtype=np.int32).reshape(-1), dtype=torch.int32, device=dev.device)
        XF = _complex_tensor(((2 if prec == PREC_FP32S else 1) * len(desc), nR, nw * nw), prec, dev.device)
        st = _lib.load().wbg_r2k_fields(_ptr(X), len(names), _ptr(dev.geom_tensors()['iR']), nR, nw, _ptr(fd),
                                        len(desc), _ptr(dev.wcc_tensor(True)), ctypes.byref(lat), prec, _ptr(XF),
                                        _stream())
        _lib.check(st, "wbg_r2k_fields")
        dev._cache[ck] = (XF, index, len(desc), fd)
    return dev._cache[ck]


def r2k(dev, dKs, NKFFT, quantities, with_H, prec, out=None, workspace=None, phases=None, block_start=0,
        lower=False, cols=None):
    """Run the R->k stage for a batch of blocks; returns (fields, index, nF, keep-alive).
    prec: False/True (FP32/FP64) or PREC_DF64 (double-float, complex128-sized slots).
    phases: optional device tables from DeviceSystem.grid_phases (then block_start indexes them).
    lower: compute only the lower triangle of the Hermitian fields (wbg_r2k_columns); their
    upper triangle is left unwritten for the consumers to mirror."""
    prec = _prec(prec)
    NKFFT = [int(n) for n in NKFFT]
    XF, index, nF, _ = field_arrays(dev, quantities, with_H, prec)
    nb = len(dKs)
    nw = dev.nw
    nk = int(np.prod(NKFFT))
    geo = r2k_geometry(dev, NKFFT)
    lib = _lib.load()
    ws = ctypes.c_size_t(0)
    _lib.check(lib.wbg_r2k_workspace_size(ctypes.byref(geo), nF, nb, prec, ctypes.byref(ws)),
               "wbg_r2k_workspace_size")
    if workspace is None or workspace.numel() < ws.value:
        workspace = torch.empty(int(ws.value), dtype=torch.uint8, device=dev.device)
    if out is None:
        out = _complex_tensor((nb * nk, nF, nw, nw), prec, dev.device)
    ph = []
    if phases is not None:
        for t in phases:
            sub = t[block_start:block_start + nb]
            ph += [sub, sub]
    else:
        for p in dev.geom.phases(dKs, NKFFT):  # page-locked staging so the upload does not stall the host
            if prec in DF64_PRECS:
                host = torch.from_numpy(_df64_pairs(p)).pin_memory()
            else:
                host = torch.from_numpy(p.astype(np.complex128 if prec == PREC_FP64 else np.complex64)).pin_memory()
            ph.append(host.to(dev.device, non_blocking=True))
            ph.append(host)  # keep the staging buffer alive until the copy has run
    gt = dev.geom_tensors()
    name = {PREC_FP32: 'r2k_fp32', PREC_FP32S: 'r2k_fp32', PREC_FP64: 'r2k_fp64', PREC_DF64: 'r2k_df64',
            PREC_DF64C: 'r2k_df64c'}[prec]
    common = (_ptr(gt['pair_start']), _ptr(gt['r2']), _ptr(gt['slice_start']), _ptr(gt['pair_r1']),
              _ptr(gt['slice_r0']), _ptr(ph[0]), _ptr(ph[2]), _ptr(ph[4]), nb, prec, _ptr(workspace),
              ctypes.c_size_t(workspace.numel()), _ptr(out), ctypes.byref(geo), _stream())
    if lower or cols is not None:
        if cols is None:
            cols, _ = column_list(dev, quantities, with_H, True)
        st = _timed(name, lib.wbg_r2k_columns, _ptr(XF), nF, _ptr(cols), cols.numel(), *common)
        _lib.check(st, "wbg_r2k_columns")
    else:
        st = _timed(name, lib.wbg_r2k, _ptr(XF), nF, *common)
        _lib.check(st, "wbg_r2k")
    return out, index, nF, (ph, workspace)


def eigh(Hfields, strideH, nw, nk, E=None, U=None, mode=1, work=None, flag=None):
    """Batched eigensolver (wbg_eigh_batched).  mode 1: FP64 throughout, U complex128;
    mode 0: FP64 solve, FP32 back-transform; mode 2: double-float solve, FP32 back-transform;
    mode 3: as 2 with double-float H (U complex64 in modes 0, 2, 3).  mode | EIGH_LOWER: H is
    read from its lower triangle."""
    lib = _lib.load()
    dev = Hfields.device
    ws = ctypes.c_size_t(0)
    _lib.check(lib.wbg_eigh_workspace_size(nw, nk, ctypes.byref(ws)), "wbg_eigh_workspace_size")
    if work is None or work.numel() < ws.value:
        work = torch.empty(int(ws.value), dtype=torch.uint8, device=dev)
    if E is None:
        E = torch.empty((nk, nw), dtype=torch.float64, device=dev)
    if U is None and not mode & EIGH_VALUES:
        U = torch.empty((nk, nw, nw), dtype=torch.complex128 if (mode & 3) == 1 else torch.complex64, device=dev)
    if flag is None:
        flag = torch.zeros(1, dtype=torch.int32, device=dev)
    st = _timed('eigh', lib.wbg_eigh_batched, _ptr(Hfields), strideH, nw, nk, _ptr(E),
                None if U is None else _ptr(U), nw * nw, int(mode), _ptr(work), ctypes.c_size_t(work.numel()),
                _ptr(flag), _stream())
    _lib.check(st, "wbg_eigh_batched")
    return E, U, flag


def rotate(U, fields, nFin, sel, herm, nw, nk, fp64, out=None):
    """wbg_rotate: fp64 1 (complex128), 0 (complex64) or 2 (double-float U and fields stored in
    complex128-sized slots, products in double-float, output complex64)."""
    lib = _lib.load()
    dev = U.device
    cdt = torch.complex128 if fp64 == 1 else torch.complex64
    if out is None:
        out = torch.empty((nk, len(sel), nw, nw), dtype=cdt, device=dev)
    key = (tuple(sel), tuple(herm), str(dev))
    if key not in _INDEX_CACHE:
        _INDEX_CACHE[key] = (torch.tensor(sel, dtype=torch.int32, device=dev),
                             torch.tensor(herm, dtype=torch.int32, device=dev))
    s, h = _INDEX_CACHE[key]
    st = _timed('rotate', lib.wbg_rotate, _ptr(U), nw * nw, _ptr(fields), nFin, _ptr(s), _ptr(h), len(sel), _ptr(out), nw, nk,
                        int(fp64), _stream())
    _lib.check(st, "wbg_rotate")
    return out, (s, h)


def band_data(dev, dKs, NKFFT, quantities, precision='fp64', phases=None, block_start=0, ws=None):
    """Stages 1-3 for a batch of blocks.  precision 'fp64': everything in FP64;
    'mixed': H(k) transform and eigh in double-float, the other fields and the rotation in FP32.
    All per-batch arrays live in persistent buffers of `dev` (reused by the next call: consume
    the returned BandData before calling again).  `phases` maps a precision code to the tables
    of DeviceSystem.grid_phases; `block_start` is the index of dKs[0] in that grid.  `ws`: the
    Workspace holding the per-batch arrays (default: the system's own), one per concurrent run."""
    require_cuda()
    quantities = set(quantities)
    if 'O' in quantities:
        quantities.discard('Od')  # a full rotation also serves diagonal-only readers
    nw = dev.nw
    NKFFT = [int(n) for n in NKFFT]
    nk = int(np.prod(NKFFT))
    nb = len(dKs)
    nkt = nb * nk
    keep = []
    ph = (lambda p: None if phases is None else phases.get(_input_prec(p)))
    arena = ws if ws is not None else dev
    flag = arena.buffer('flag', (1,), torch.int32)
    flag.zero_()

    def fields_for(q, with_H, prec, name, lower=False, wsname='r2k_ws', cols=None):
        _, _, nF, _ = field_arrays(dev, q, with_H, prec)
        out = arena.buffer(name, (nkt, nF, nw, nw), torch.complex64 if prec in C64_PRECS else torch.complex128)
        geo = r2k_geometry(dev, NKFFT)
        wsz = ctypes.c_size_t(0)
        _lib.check(_lib.load().wbg_r2k_workspace_size(ctypes.byref(geo), nF, nb, prec, ctypes.byref(wsz)),
                   "wbg_r2k_workspace_size")
        work = arena.buffer(wsname, (int(wsz.value),), torch.uint8)
        return r2k(dev, dKs, NKFFT, q, with_H, prec, out=out, workspace=work, phases=ph(prec),
                   block_start=block_start, lower=lower, cols=cols)

    E = arena.buffer('E', (nkt, nw), torch.float64)
    ews = ctypes.c_size_t(0)
    _lib.check(_lib.load().wbg_eigh_workspace_size(nw, nkt, ctypes.byref(ews)), "wbg_eigh_workspace_size")
    ework = arena.buffer('eigh_ws', (int(ews.value),), torch.uint8)
    if precision == 'fp64':
        fields, index, nF, k1 = fields_for(quantities, True, PREC_FP64, 'fields')
        keep.append(k1)
        U = arena.buffer('U', (nkt, nw, nw), torch.complex128)
        E, U, flag = eigh(fields, nF * nw * nw, nw, nkt, E=E, U=U, mode=1, work=ework, flag=flag)
        fp64_fields = True
    elif precision == 'mixed':
        # lower triangles of the Hermitian fields only: exactly Hermitian, half the transform
        lowerH = 'Ham' in dev.hermitian_bases()  # else the eigensolver symmetrises the full H(k)
        Hf, _, _, k0 = fields_for(set(), True, PREC_DF64, 'fields_H', lower=lowerH)
        keep.append(k0)
        wide = nw > MIXED_FP32_ROTATION_MAX_NW and bool(quantities)
        if wide:  # double-float vectors, fields and rotation; Xbar rounded to complex64 once
            U = arena.buffer('Udf', (nkt, nw, nw), torch.complex128)
            mode = 3 | (EIGH_LOWER if lowerH else 0) | EIGH_PRECISE_VECTORS | EIGH_DF64_VECTORS
        else:
            U = arena.buffer('U32', (nkt, nw, nw), torch.complex64)
            refine = MIXED_EIGH_REFINE and MIXED_EIGH_REFINE_NW[0] < nw <= MIXED_EIGH_REFINE_NW[1]
            bits = EIGH_REFINE if refine else MIXED_EIGH_BITS
            mode = 3 | (EIGH_LOWER if lowerH else 0) | bits
        if quantities:
            # the FP32 fields do not depend on the eigensolver: their transform runs on a side
            # stream next to the QL iteration (a few warps per SM, latency-bound), started once
            # the tridiagonalisation (which fills the SMs' shared memory) is done.  A fresh system's
            # upload of the other R-space matrices and their weights go ahead on the side stream
            # right away (after the main stream's upload of H, which they also read).
            main = torch.cuda.current_stream()
            side = arena.side_stream()
            fprec = PREC_DF64 if wide else MIXED_FIELDS_PREC
            need = {_input_prec(fprec)}
            if not wide and MIXED_DF64_QUANTITIES & set(quantities):
                need.add(PREC_DF64)
            if any(('XF', tuple(sorted(quantities)), False, p) not in dev._cache for p in need):
                h_ready = torch.cuda.Event()
                h_ready.record(main)
                with torch.cuda.stream(side):
                    side.wait_event(h_ready)
                    for p in need:
                        field_arrays(dev, quantities, False, p)
            eigh(Hf, nw * nw, nw, nkt, E=E, U=U, mode=mode | EIGH_STAGE1, work=ework, flag=flag)
            tridiag_done = torch.cuda.Event()
            tridiag_done.record(main)
            with torch.cuda.stream(side):
                side.wait_event(tridiag_done)
                dfq = MIXED_DF64_QUANTITIES & set(quantities) if not wide else set()
                if dfq and fprec != PREC_DF64C:
                    # the fields of dfq in double-float (rounded to complex64), the rest in fprec,
                    # into one array: two column lists over the same field layout
                    cdf, crest = split_columns(dev, quantities, False, True, dfq)
                    fields, index, nF, k1 = fields_for(quantities, False, PREC_DF64C, 'fields', cols=cdf,
                                                       wsname='r2k_ws_fields')
                    if crest.numel():
                        _, _, _, k1b = fields_for(quantities, False, fprec, 'fields', cols=crest,
                                                  wsname='r2k_ws_fields2')
                        keep.append(k1b)
                else:
                    fields, index, nF, k1 = fields_for(quantities, False, fprec, 'fields', lower=True,
                                                       wsname='r2k_ws_fields')
            E, U, flag = eigh(Hf, nw * nw, nw, nkt, E=E, U=U, mode=mode | EIGH_STAGE2, work=ework, flag=flag)
            main.wait_stream(side)
            keep.append(k1)
            lower_in = column_list(dev, quantities, False, True)[1]
        else:  # energies only (DOS-type calculators): no band-basis fields
            E, U, flag = eigh(Hf, nw * nw, nw, nkt, E=E, U=U, mode=mode, work=ework, flag=flag)
            fields, index, nF, lower_in = None, {}, 0, []
        fp64_fields = False
        rot_prec = 2 if wide else 0
    else:
        raise ValueError(f"unknown precision mode {precision!r}")
    sel, herm, bindex = [], [], {}
    for q in QUANTITY_ORDER:
        if q in quantities:
            bindex[q] = len(sel)
            n = QUANTITIES[q]['ncomp']
            sel += list(range(index[q], index[q] + n))
            herm += [QUANTITIES[q]['herm']] * n
    if not fp64_fields:
        # mirrored (exactly Hermitian) inputs: flag them, and keep the Hermitian part of their
        # rotation, which drops only the FP32 rounding noise of U^dagger X U
        herm = [(h or 1) | 4 if lower_in[f] else h for f, h in zip(sel, herm)]
    if sel:
        Xb = arena.buffer('Xbar', (nkt, len(sel), nw, nw), torch.complex128 if fp64_fields else torch.complex64)
        Xbar, k2 = rotate(U, fields, nF, sel, herm, nw, nkt, 1 if fp64_fields else rot_prec, out=Xb)
        keep.append(k2)
    else:
        Xbar = None
    if 'O' in bindex:
        bindex['Od'] = bindex['O']
    # mixed path: V and A come from mirrored (exactly Hermitian) inputs and their rotation keeps
    # the Hermitian part, so Xbar's V and A blocks are exactly Hermitian
    herm_out = (not fp64_fields) and all(lower_in[index[q] + c] for q in ('V', 'A') if q in index
                                         for c in range(3))
    bd = BandData(E, U, Xbar, bindex, nb, nk, nw, fp64_fields, hermitian=herm_out)
    bd._keep = keep
    bd._flag = flag
    return bd


class _GraphEntry:
    """A captured band_data launch sequence: the graph, the BandData whose buffers it writes, its
    fixed phase-table inputs, the workspace generation it was captured at and its system."""

    def __init__(self, graph, bd, tabs, generation, dev):
        self.graph, self.bd, self.tabs, self.generation, self.dev = graph, bd, tabs, generation, dev
        self.replays = 0


def phase_precs(precision):
    """Phase-table precisions band_data reads for `precision` (the grid tables a run precomputes)."""
    if precision == 'fp64':
        return [PREC_FP64]
    return sorted({PREC_DF64, _input_prec(MIXED_FIELDS_PREC)})


def _graph_precs(quantities, precision):
    """Phase-table precisions that band_data reads for `precision`."""
    if precision == 'fp64':
        return [PREC_FP64]
    fp = _input_prec(MIXED_FIELDS_PREC)
    return sorted({PREC_DF64, fp}) if quantities else [PREC_DF64]


def _fill_phase_inputs(dev, tabs, dKs, NKFFT, phases, block_start):
    """Copy a batch's per-axis phase tables into a graph's fixed inputs on the current stream:
    a device-to-device copy from the grid's resident tables (`phases`, rows block_start..), or
    the tables of the shifts `dKs` built on the host when the grid has none."""
    nb = len(dKs)
    host = None
    for p, dst in tabs.items():
        if phases is not None and p in phases:
            for d, t in zip(dst, phases[p]):
                d.copy_(t[block_start:block_start + nb], non_blocking=True)
            continue
        if host is None:
            host = dev.geom.phases(dKs, NKFFT)
        for d, h in zip(dst, host):
            a = _df64_pairs(h) if p == PREC_DF64 else h.astype(np.complex128 if p == PREC_FP64 else np.complex64)
            d.copy_(torch.from_numpy(a))


def band_data_graphed(dev, dKs, NKFFT, quantities, precision='fp64', phases=None, block_start=0, ws=None,
                      more=True):
    """band_data (stages 1-3) replayed from a CUDA graph of its launch sequence.

    One graph per (FFT grid, blocks per batch, quantities, precision) and workspace.  The first
    batch of a shape runs plain launches (it also fills the host-side caches: R-space fields,
    column lists, field selections); the second is run plain once more on the graph's fixed
    phase-table inputs and captured; later batches copy their phase tables into those inputs and
    replay the graph, so a batch costs a few host calls instead of one Python dispatch per kernel.
    The graph writes the same workspace buffers as band_data, so results are bit-identical to it.
    A graph is dropped when its workspace reallocates a buffer (Workspace.generation) or serves
    another system.  ``more``: whether the caller will issue further batches of this shape on this
    workspace; a capture (which synchronises the device) is made only then.  Stage timers
    (set_timer) need plain launches: with a timer set this is band_data itself.  The returned
    BandData is valid until the next batch on the same workspace, as for band_data."""
    if _TIMER is not None:
        return band_data(dev, dKs, NKFFT, quantities, precision, phases=phases, block_start=block_start, ws=ws)
    arena = ws if ws is not None else dev.workspace()
    NKFFT = [int(n) for n in NKFFT]
    quantities = frozenset(quantities)
    nb = len(dKs)
    key = (tuple(NKFFT), nb, quantities, precision)
    ent = arena.graphs.get(key)
    if ent is not None and (ent.dev is not dev or ent.generation != arena.generation):
        del arena.graphs[key]
        ent = None
    if ent is not None:
        _fill_phase_inputs(dev, ent.tabs, dKs, NKFFT, phases, block_start)
        ent.graph.replay()
        ent.replays += 1
        return copy.copy(ent.bd)
    seen = arena.__dict__.setdefault('_graph_seen', set())
    if (key, id(dev)) not in seen or not more:
        seen.add((key, id(dev)))
        return band_data(dev, dKs, NKFFT, quantities, precision, phases=phases, block_start=block_start, ws=ws)
    # capture: fixed inputs, one plain run on them (this batch's result; every buffer at its final
    # size), then the same call captured
    g = dev.geom
    tabs = {}
    for p in _graph_precs(quantities, precision):
        lst = []
        for d in range(3):
            shape = (nb, NKFFT[d], int(g.nr[d]))
            if p == PREC_DF64:
                lst.append(arena.buffer(f'graph_ph{p}_{d}', shape + (4,), torch.float32))
            else:
                lst.append(arena.buffer(f'graph_ph{p}_{d}', shape, torch.complex128 if p == PREC_FP64 else
                                        torch.complex64))
        tabs[p] = lst
    _fill_phase_inputs(dev, tabs, dKs, NKFFT, phases, block_start)
    bd = band_data(dev, dKs, NKFFT, quantities, precision, phases=tabs, block_start=0, ws=ws)
    generation = arena.generation
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, capture_error_mode='relaxed'):
        gbd = band_data(dev, dKs, NKFFT, quantities, precision, phases=tabs, block_start=0, ws=ws)
    if arena.generation != generation:  # band_data grew a buffer while capturing: do not keep it
        raise RuntimeError("band_data_graphed: workspace changed during capture")
    arena.graphs[key] = _GraphEntry(graph, gbd, tabs, generation, dev)
    return bd


def energies(dev, dKs, NKFFT, precision='fp64', out=None, phases=None, block_start=0, ws=None):
    """Eigenvalues of H(k) only (np.linalg.eigvalsh) for a batch of blocks: (nblocks*nk, nw)
    float64 written to `out` when given.  FP64 ('fp64') or double-float ('mixed') transform and
    tridiagonal QL, no eigenvectors.  Returns (E, flag)."""
    require_cuda()
    nw = dev.nw
    NKFFT = [int(n) for n in NKFFT]
    nkt = len(dKs) * int(np.prod(NKFFT))
    arena = ws if ws is not None else dev
    flag = arena.buffer('flag_E', (1,), torch.int32)
    flag.zero_()
    if precision == 'fp64':
        prec, lower, mode = PREC_FP64, False, 1
    elif precision == 'mixed':
        lower = 'Ham' in dev.hermitian_bases()
        prec, mode = PREC_DF64, 3 | (EIGH_LOWER if lower else 0)
    else:
        raise ValueError(f"unknown precision mode {precision!r}")
    _, _, nF, _ = field_arrays(dev, set(), True, prec)
    Hf = arena.buffer('fields_H', (nkt, nF, nw, nw), torch.complex128)
    geo = r2k_geometry(dev, NKFFT)
    wsz = ctypes.c_size_t(0)
    _lib.check(_lib.load().wbg_r2k_workspace_size(ctypes.byref(geo), nF, len(dKs), prec, ctypes.byref(wsz)),
               "wbg_r2k_workspace_size")
    work = arena.buffer('r2k_ws', (int(wsz.value),), torch.uint8)
    Hf, _, _, keep = r2k(dev, dKs, NKFFT, set(), True, prec, out=Hf, workspace=work,
                         phases=None if phases is None else phases.get(prec), block_start=block_start, lower=lower)
    ews = ctypes.c_size_t(0)
    _lib.check(_lib.load().wbg_eigh_workspace_size(nw, nkt, ctypes.byref(ews)), "wbg_eigh_workspace_size")
    ework = arena.buffer('eigh_ws', (int(ews.value),), torch.uint8)
    E = out if out is not None else arena.buffer('E', (nkt, nw), torch.float64)
    E, _, flag = eigh(Hf, nF * nw * nw, nw, nkt, E=E, U=None, mode=mode | EIGH_VALUES, work=ework, flag=flag)
    del keep
    return E, flag


class TetraCorners:
    """Corner energies of the tetrahedron method for a run over `grid` (grid/tetrahedron.py
    TetraWeightsParal, data_K/data_K_R.py:121-141).  The corners k +- delta/2 of every k-point
    (delta = 1/(NKdiv NKFFT)) are the dense grid shifted by +delta/2; corner block c is the FFT
    grid at shift (c + 1/2) delta.  The corner blocks that the run's blocks touch (i and i-1 per
    axis) are evaluated once and stay resident: Ec (ncorner*nk, nw) float64, slot[flat corner
    block] = its row (-1: not evaluated)."""

    def __init__(self, dev, grid, blocks=None, precision='fp64', ws=None, batch=None):
        div, fft = np.array(grid.div, dtype=int), np.array(grid.FFT, dtype=int)
        self.grid = _lib.TetraGrid((ctypes.c_int * 3)(*div.tolist()), (ctypes.c_int * 3)(*fft.tolist()), 0)
        self.nblocks_total = int(np.prod(div))
        blocks = np.arange(self.nblocks_total) if blocks is None else np.asarray(blocks, dtype=int)
        idx = np.stack(np.unravel_index(blocks, div), axis=-1)
        need = set()
        for s in range(8):
            c = idx.copy()
            for a in range(3):
                if not (s >> (2 - a)) & 1:
                    c[:, a] = (c[:, a] - 1) % div[a]
            need.update(np.ravel_multi_index(c.T, div).tolist())
        cb = np.array(sorted(need), dtype=int)
        slot = -np.ones(self.nblocks_total, dtype=np.int32)
        slot[cb] = np.arange(len(cb), dtype=np.int32)
        self.slot = torch.from_numpy(slot).to(dev.device)
        shifts = (np.stack(np.unravel_index(cb, div), axis=-1) + 0.5) / (div * fft)[None, :]
        nk = int(np.prod(fft))
        nw = dev.nw
        self.Ec = torch.empty((len(cb) * nk, nw), dtype=torch.float64, device=dev.device)
        prec = PREC_FP64 if precision == 'fp64' else PREC_DF64
        phases = {prec: dev.grid_phases(shifts, fft, prec)}
        if batch is None:
            from .run import choose_batch
            batch = choose_batch(nw, nk, len(cb), set(), precision)
        self.flags = []  # QL convergence flags, read by check() (no synchronisation here)
        for i0 in range(0, len(cb), batch):
            n = min(batch, len(cb) - i0)
            _, flag = energies(dev, shifts[i0:i0 + n], fft, precision, out=self.Ec[i0 * nk:(i0 + n) * nk],
                               phases=phases, block_start=i0, ws=ws)
            self.flags.append(flag.clone())
        self.device = dev.device

    @staticmethod
    def nbytes(grid, nblocks, nw):
        """Upper bound of the resident corner energies for a run over `nblocks` blocks."""
        ncorner = min(int(np.prod(grid.div)), 8 * int(nblocks))
        return ncorner * int(np.prod(grid.FFT)) * nw * 8

    def check(self):
        if any(int(f.item()) != 0 for f in self.flags):
            raise RuntimeError("wbg_eigh_batched: QL iteration did not converge for some corner k-point")

    def attach(self, bd, block_ids):
        """Give a batch's BandData its corner context (block_ids: flat division-grid indices)."""
        bd.tetra = self
        bd.tetra_blocks = torch.tensor(np.asarray(block_ids, dtype=np.int32), device=self.device)
        bd.tetra_sel = {}
        return bd

    def selection(self, bd, EF0, EF1, degen_thresh, sea):
        """wbg_tetra_select for a batch (cached per window on the BandData)."""
        key = (float(EF0), float(EF1), float(degen_thresh), int(sea))
        if key not in bd.tetra_sel:
            sel = torch.empty((bd.nk_total, bd.nw), dtype=torch.int8, device=self.device)
            st = _timed('tetra_select', _lib.load().wbg_tetra_select, _ptr(bd.E), _ptr(self.Ec), _ptr(self.slot),
                        _ptr(bd.tetra_blocks), bd.nblocks, ctypes.byref(self.grid), bd.nw, ctypes.c_double(EF0),
                        ctypes.c_double(EF1), ctypes.c_double(degen_thresh), int(sea), _ptr(sel), _stream())
            _lib.check(st, "wbg_tetra_select")
            bd.tetra_sel[key] = sel
        return bd.tetra_sel[key]


class BlockCorners(TetraCorners):
    """Corner energies of arbitrary blocks, e.g. refined K-points whose cell differs from the
    grid's (data_K/data_K_R.py:121-141 with Kpoint.dK_fullBZ of each K-point): block b at shift
    dK_b with cell c_b = dK_block / NKFFT gets the 8 grids at dK_b + (+-c_b/2 per axis), corner
    s = 4 sx + 2 sy + sz (0: minus side) at Ecorner row 8 b + s; the kernels address them through
    wbg_tetra_grid.per_block.  Blocks are identified by their position in `shifts`."""

    def __init__(self, dev, shifts, cells, NKFFT, precision='fp64', ws=None):
        fft = np.array(NKFFT, dtype=int) * np.ones(3, dtype=int)
        self.grid = _lib.TetraGrid((ctypes.c_int * 3)(1, 1, 1), (ctypes.c_int * 3)(*fft.tolist()), 1)
        shifts, cells = np.asarray(shifts, dtype=float), np.asarray(cells, dtype=float)
        nb, nk, nw = len(shifts), int(np.prod(fft)), dev.nw
        sgn = np.array([[(s >> (2 - a)) & 1 for a in range(3)] for s in range(8)], dtype=float) - 0.5
        corner_shifts = (shifts[:, None, :] + sgn[None, :, :] * cells[:, None, :]).reshape(-1, 3)
        self.Ec = torch.empty((len(corner_shifts) * nk, nw), dtype=torch.float64, device=dev.device)
        self.slot = torch.arange(nb, dtype=torch.int32, device=dev.device)
        from .run import choose_batch
        batch = choose_batch(nw, nk, len(corner_shifts), set(), precision)
        self.flags = []
        for i0 in range(0, len(corner_shifts), batch):
            n = min(batch, len(corner_shifts) - i0)
            _, flag = energies(dev, corner_shifts[i0:i0 + n], fft, precision, out=self.Ec[i0 * nk:(i0 + n) * nk],
                               ws=ws)
            self.flags.append(flag.clone())
        self.device = dev.device


def device_flags(clear=True):
    """Library device error word (wbg_device_flags); nonzero after a tensor-core wait timed out."""
    v = ctypes.c_uint(0)
    _lib.check(_lib.load().wbg_device_flags(ctypes.byref(v), int(clear)), "wbg_device_flags")
    return int(v.value)


def _flag_word(v):
    if v & 1:
        raise RuntimeError("wbg_eigh_batched: QL iteration did not converge for some k-point")
    if v & 4:
        warnings.warn("wbg_eigh_batched (refined): a cluster of more than 8 close eigenvalues was "
                      "re-diagonalised 8 at a time, or a matrix did not settle in two refinement steps; "
                      "its eigenpairs may keep FP32 accuracy", RuntimeWarning)


def check_flag(bd):
    _flag_word(int(bd._flag.item()))


def check_flags(flags):
    """The eigensolver flags of several batches (device int32 tensors) read in one copy: bit 0 (QL
    did not converge) raises, bit 2 (refined solve: a cluster wider than 8) warns."""
    if flags:
        v = torch.cat([f.reshape(-1) for f in flags]).cpu().numpy()
        _flag_word(int(np.bitwise_or.reduce(v.astype(np.int64))))
