"""Autotuner of the kernels' launch shapes (no counterpart in the reference, whose numpy calls
have no launch shapes).

The library keeps a process-wide table of launch shapes per (parameter, variant, num_wann)
(``wbg_tune_set`` / ``wbg_tune_get`` in include/wbgpu.h); 0 means the built-in occupancy
heuristic.  This module measures the candidates that the library lists for a num_wann
(``wbg_tune_candidates``: only shapes that fit the kernels' launch limits) on a synthetic batch
with CUDA events, keeps the fastest per parameter (coordinate descent: each parameter timed with
the others at their best so far), writes it into the table, and caches the choices per device in
a JSON file so that later processes apply them without measuring.

Parameters: the eigensolver's three group sizes (tridiagonalisation, QL sweep, inverse
iteration + back-transform) per eigh mode (FP64 ``mode 1``, double-float ``mode 3``), and for the
rotation the k-points per block of the CUDA-core tiled kernel and, at nw = 32 in FP32, the engine
(tensor cores or CUDA cores).  The eigensolver shapes and the tiled-rotation shape do not change
results (every matrix / k-point is computed by the same code whatever the grouping); the rotation
engine changes FP32 rounding within the FP32 path's error budget.
"""
import ctypes
import json
import os

import numpy as np

from . import _lib

EIGH_TRIDIAG_GROUP, EIGH_QL_BLOCK, EIGH_VECTORS_GROUP, ROTATE_KPOINTS, ROTATE_ENGINE, KUBO_ENGINE = range(6)
PARAM_NAMES = {EIGH_TRIDIAG_GROUP: 'eigh_tridiag_group', EIGH_QL_BLOCK: 'eigh_ql_block',
               EIGH_VECTORS_GROUP: 'eigh_vectors_group', ROTATE_KPOINTS: 'rotate_kpoints',
               ROTATE_ENGINE: 'rotate_engine', KUBO_ENGINE: 'kubo_engine'}
EIGH_PARAMS = (EIGH_TRIDIAG_GROUP, EIGH_QL_BLOCK, EIGH_VECTORS_GROUP)
ROTATE_PARAMS = (ROTATE_KPOINTS, ROTATE_ENGINE)
# eigh mode and rotation variant (fp64 flag) of each precision of run()
PRECISE_VECTORS = 64  # wbg_eigh_batched mode bit WBG_EIGH_PRECISE_VECTORS
PRECISION_VARIANTS = {'fp64': (1, 1), 'mixed': (3 | PRECISE_VECTORS, 0)}


def eigh_variant(mode):
    """The tuning table's eigensolver variant of a wbg_eigh_batched mode: mode & 3, except the
    double-float solve with its double-float back-transform (4) and the FP64 solve with the FP64
    back-transform rounded to FP32 (1, the launch shapes of mode 1)."""
    if mode & PRECISE_VECTORS:
        return {0: 1, 1: 1, 2: 4, 3: 4}[mode & 3]
    return mode & 3


def candidates(param, nw, variant):
    """Launch-shape values the library accepts for (param, nw, variant)."""
    arr = (ctypes.c_int * 32)()
    n = ctypes.c_int(0)
    _lib.check(_lib.load().wbg_tune_candidates(param, nw, variant, arr, 32, ctypes.byref(n)), "wbg_tune_candidates")
    return list(arr[:n.value])


def set_value(param, nw, variant, value):
    """Write one table entry (0: the built-in heuristic); ValueError for a value the kernels
    do not accept."""
    _lib.check(_lib.load().wbg_tune_set(param, nw, variant, int(value)), "wbg_tune_set")


def get_value(param, nw, variant):
    v = ctypes.c_int(0)
    _lib.check(_lib.load().wbg_tune_get(param, nw, variant, ctypes.byref(v)), "wbg_tune_get")
    return int(v.value)


def reset(nws=range(1, 129)):
    """Every entry of the given num_wann back to the built-in heuristics."""
    for nw in nws:
        for p in EIGH_PARAMS:
            for v in range(6):
                set_value(p, nw, v, 0)
        for p in ROTATE_PARAMS:
            for v in (0, 1):
                set_value(p, nw, v, 0)
    set_value(KUBO_ENGINE, 1, 0, 0)


def coordinate_descent(params, time_fn, apply_fn, rounds=1):
    """Pick one value per parameter: `params` maps a parameter to its candidate list,
    `time_fn()` measures the current configuration, `apply_fn(param, value)` sets one value.
    Each parameter in turn tries all its candidates with the others fixed and keeps the fastest
    (ties: the first measured).  Returns ({param: value}, {param: {value: time}})."""
    best = {}
    timings = {}
    for _ in range(rounds):
        for p, cands in params.items():
            if not cands:
                continue
            ts = {}
            for c in cands:
                apply_fn(p, c)
                ts[c] = float(time_fn())
            pick = min(ts, key=lambda c: (ts[c], cands.index(c)))
            apply_fn(p, pick)
            best[p] = pick
            timings[p] = ts
    return best, timings


def _time_ms(torch, fn, reps):
    fn()  # warm-up (also the first launch's attribute setting)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    e.synchronize()
    return s.elapsed_time(e) / reps


def default_batch(nw, nk=None):
    """Matrices per timing launch: about the work of 16 384 matrices at nw = 32."""
    if nk is None:
        nk = int(16384 * (32.0 / nw) ** 3)
    return int(min(max(nk, 1024), 32768))


def _eigh_runner(nw, mode, nk, seed, device):
    """A closure launching wbg_eigh_batched on nk seeded random Hermitian matrices."""
    import torch
    from . import engine
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw))
    H = 0.5 * (A + np.conj(np.swapaxes(A, 1, 2)))
    if (mode & 3) == 3:
        Hd = torch.from_numpy(engine._df64_pairs(H)).to(device)
    else:
        Hd = torch.from_numpy(H).to(device)
    E = torch.empty((nk, nw), dtype=torch.float64, device=device)
    U = torch.empty((nk, nw, nw), dtype=torch.complex128 if (mode & 3) == 1 else torch.complex64, device=device)
    flag = torch.zeros(1, dtype=torch.int32, device=device)
    ws = ctypes.c_size_t(0)
    lib = _lib.load()
    _lib.check(lib.wbg_eigh_workspace_size(nw, nk, ctypes.byref(ws)), "wbg_eigh_workspace_size")
    work = torch.empty(int(ws.value), dtype=torch.uint8, device=device)

    def run():
        _lib.check(lib.wbg_eigh_batched(engine._ptr(Hd), nw * nw, nw, nk, engine._ptr(E), engine._ptr(U), nw * nw,
                                        int(mode), engine._ptr(work), ctypes.c_size_t(work.numel()),
                                        engine._ptr(flag), engine._stream()), "wbg_eigh_batched")
    return run


def time_eigh(nw, mode, nk=None, reps=5, seed=0, device='cuda'):
    """ms per wbg_eigh_batched launch of `default_batch(nw, nk)` matrices with the table's
    current shapes."""
    import torch
    return _time_ms(torch, _eigh_runner(nw, mode, default_batch(nw, nk), seed, device), reps)


def tune_eigh(nw, mode, nk=None, reps=3, seed=0, device='cuda'):
    """Tune the eigensolver's group sizes for (nw, eigh_variant(mode)) on nk random Hermitian
    matrices; the table holds the choice afterwards.  Returns ({name: value}, {name: {value: ms}})."""
    import torch
    variant = eigh_variant(mode)
    run = _eigh_runner(nw, mode, default_batch(nw, nk), seed, device)
    params = {p: candidates(p, nw, variant) for p in EIGH_PARAMS}
    params = {p: c for p, c in params.items() if len(c) > 1}
    best, timings = coordinate_descent(params, lambda: _time_ms(torch, run, reps),
                                       lambda p, v: set_value(p, nw, variant, v))
    return ({PARAM_NAMES[p]: v for p, v in best.items()},
            {PARAM_NAMES[p]: t for p, t in timings.items()})


def tune_rotate(nw, fp64, nk=None, nfields=9, reps=3, seed=0, device='cuda'):
    """Tune the rotation for (nw, fp64) on nk random k-points of `nfields` fields (the AHC field
    count of the mixed path by default); the table holds the choice afterwards."""
    import torch
    from . import engine
    params = {p: candidates(p, nw, int(bool(fp64))) for p in ROTATE_PARAMS}
    params = {p: c for p, c in params.items() if len(c) > 1}
    if not params:
        return {}, {}
    nk = default_batch(nw, nk)
    rng = np.random.default_rng(seed)
    cdt = torch.complex128 if fp64 else torch.complex64
    U = torch.from_numpy(rng.standard_normal((nk, nw, nw)) + 1j * rng.standard_normal((nk, nw, nw))).to(device, cdt)
    X = torch.from_numpy(rng.standard_normal((nk, nfields, nw, nw)) +
                         1j * rng.standard_normal((nk, nfields, nw, nw))).to(device, cdt)
    out = torch.empty_like(X)
    sel = torch.arange(nfields, dtype=torch.int32, device=device)
    herm = torch.ones(nfields, dtype=torch.int32, device=device)
    lib = _lib.load()

    def run():
        _lib.check(lib.wbg_rotate(engine._ptr(U), nw * nw, engine._ptr(X), nfields, engine._ptr(sel),
                                  engine._ptr(herm), nfields, engine._ptr(out), nw, nk, int(bool(fp64)),
                                  engine._stream()), "wbg_rotate")

    variant = int(bool(fp64))
    best, timings = coordinate_descent(params, lambda: _time_ms(torch, run, reps),
                                       lambda p, v: set_value(p, nw, variant, v))
    return ({PARAM_NAMES[p]: v for p, v in best.items()},
            {PARAM_NAMES[p]: t for p, t in timings.items()})


# ---------------------------------------------------------------------------------- cache file
def cache_path():
    """JSON file of tuned shapes: $WBGPU_TUNE_CACHE, else ~/.cache/wbgpu/tune.json."""
    p = os.environ.get('WBGPU_TUNE_CACHE')
    if p:
        return p
    return os.path.join(os.path.expanduser('~'), '.cache', 'wbgpu', 'tune.json')


def _entry_key(device_name, nw, precision):
    abi = _lib.load().wbg_abi_version()
    return f"{device_name}|abi{abi}|nw{int(nw)}|{precision}"


def load_cache(path=None):
    try:
        with open(path or cache_path()) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def save_cache(data, path=None):
    path = path or cache_path()
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + '.tmp'
    with open(tmp, 'w') as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply_entry(entry, nw, precision):
    """Write a cached {parameter name: value} entry into the library's table."""
    mode, rvariant = PRECISION_VARIANTS[precision]
    ids = {v: k for k, v in PARAM_NAMES.items()}
    for name, value in entry.items():
        p = ids[name]
        set_value(p, nw, eigh_variant(mode) if p in EIGH_PARAMS else rvariant, int(value))


def ensure(nw, precision, device='cuda', path=None, retune=False):
    """Tuned launch shapes for (num_wann, precision) on this device: applied from the cache
    file when present, else measured now (tune_eigh + tune_rotate) and saved.  Returns the
    {parameter name: value} entry."""
    import torch
    name = torch.cuda.get_device_name(torch.device(device))
    key = _entry_key(name, nw, precision)
    data = load_cache(path)
    if key in data and not retune:
        apply_entry(data[key], nw, precision)
        return data[key]
    mode, rvariant = PRECISION_VARIANTS[precision]
    entry, _ = tune_eigh(nw, mode, device=device)
    r, _ = tune_rotate(nw, rvariant, device=device)
    entry.update(r)
    data = load_cache(path)
    data[key] = entry
    save_cache(data, path)
    return entry
