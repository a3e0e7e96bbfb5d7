"""ctypes binding of libwbgpu.so (C ABI declared in include/wbgpu.h).

Status codes are turned into the exception types the reference raises for the same
kind of failure: ValueError for bad arguments / sizes, RuntimeError for CUDA errors
and eigensolver non-convergence (the reference raises RuntimeError for numerical
failures, e.g. data_K/data_K.py:239-241).
"""
import ctypes
import os

from . import build as _build

EXPORTS = ['wbg_abi_version', 'wbg_status_string', 'wbg_last_cuda_error_string', 'wbg_r2k_fields', 'wbg_r2k_workspace_size', 'wbg_r2k',
           'wbg_r2k_columns', 'wbg_ws_replicas',
           'wbg_eigh_workspace_size', 'wbg_eigh_batched', 'wbg_eigh_batched_noalloc', 'wbg_rotate', 'wbg_device_flags', 'wbg_tc_wait_limit', 'wbg_tc_wait_probe', 'wbg_berry_tabulate', 'wbg_berry_scan',
           'wbg_berry_omega', 'wbg_berry_morb', 'wbg_berry_deromega', 'wbg_kubo_workspace_size', 'wbg_kubo',
           'wbg_dynamic_ncomp', 'wbg_dynamic_workspace_size', 'wbg_dynamic', 'wbg_berry_shc',
           'wbg_berry_product', 'wbg_product_values',
           'wbg_scan_finalize', 'wbg_tetra_select', 'wbg_band_values', 'wbg_tetra_accumulate', 'wbg_probe_fma',
           'wbg_tune_candidates', 'wbg_tune_set', 'wbg_tune_get']

STATUS_OK = 0


class R2KGeom(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in
                ['nR', 'nw', 'nw2', 'nBase', 'nP', 'nU', 'N0', 'N1', 'N2', 'nk', 'nr0', 'nr1', 'nr2',
                 'rmin0', 'rmin1', 'rmin2', 'maxPairLen', 'maxSliceLen']]


class Lattice(ctypes.Structure):
    _fields_ = [('L', ctypes.c_double * 9)]


class Scan(ctypes.Structure):
    _fields_ = [('EFmin', ctypes.c_double), ('EFmax', ctypes.c_double), ('dEF', ctypes.c_double),
                ('degen_thresh', ctypes.c_double), ('nEF', ctypes.c_int), ('reserved', ctypes.c_int)]


class KuboParams(ctypes.Structure):
    _fields_ = [('EFmin', ctypes.c_double), ('EFmax', ctypes.c_double), ('kBT', ctypes.c_double),
                ('eta', ctypes.c_double), ('degen_thresh', ctypes.c_double), ('nEF', ctypes.c_int),
                ('nOmega', ctypes.c_int), ('gaussian', ctypes.c_int), ('reserved', ctypes.c_int)]


class DynamicSpec(ctypes.Structure):
    _fields_ = ([('formula', ctypes.c_int), ('external_terms', ctypes.c_int)] +
                [(n, ctypes.c_int) for n in ['V', 'A', 'W', 'dA', 'S', 'SH', 'SA', 'SHA', 'SR', 'SHR']] +
                [('sc_eta', ctypes.c_double), ('omega_min', ctypes.c_double), ('omega_max', ctypes.c_double)])


class TetraGrid(ctypes.Structure):
    _fields_ = [('div', ctypes.c_int * 3), ('fft', ctypes.c_int * 3), ('per_block', ctypes.c_int)]


class FieldIndex(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ['V', 'A', 'O', 'W', 'dA', 'dO', 'B', 'C']]


class ProductSpec(ctypes.Structure):
    _fields_ = ([('nfactors', ctypes.c_int), ('factor', ctypes.c_int * 3), ('internal_terms', ctypes.c_int),
                 ('external_terms', ctypes.c_int)] +
                [(n, ctypes.c_int) for n in ['V', 'A', 'O', 'W', 'S', 'B', 'C', 'dS']])


_P = ctypes.c_void_p
_I = ctypes.c_int
_LL = ctypes.c_longlong
_SZ = ctypes.c_size_t

_SIGS = {
    'wbg_abi_version': (_I, []),
    'wbg_status_string': (ctypes.c_char_p, [_I]),
    'wbg_last_cuda_error_string': (ctypes.c_char_p, []),
    'wbg_r2k_fields': (_I, [_P, _I, _P, _I, _I, _P, _I, _P, ctypes.POINTER(Lattice), _I, _P, _P]),
    'wbg_r2k_workspace_size': (_I, [ctypes.POINTER(R2KGeom), _I, _I, _I, ctypes.POINTER(_SZ)]),
    'wbg_r2k': (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _P, _SZ, _P, ctypes.POINTER(R2KGeom), _P]),
    'wbg_r2k_columns': (_I, [_P, _I, _P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _P, _SZ, _P,
                             ctypes.POINTER(R2KGeom), _P]),
    'wbg_eigh_workspace_size': (_I, [_I, _I, ctypes.POINTER(_SZ)]),
    'wbg_eigh_batched': (_I, [_P, _LL, _I, _I, _P, _P, _LL, _I, _P, _SZ, _P, _P]),
    'wbg_eigh_batched_noalloc': (_I, [_P, _LL, _I, _I, _P, _P, _LL, _I, _P, _P]),
    'wbg_rotate': (_I, [_P, _LL, _P, _I, _P, _P, _I, _P, _I, _I, _I, _P]),
    'wbg_device_flags': (_I, [ctypes.POINTER(ctypes.c_uint), _I]),
    'wbg_tc_wait_limit': (_I, [ctypes.c_ulonglong]),
    'wbg_tc_wait_probe': (_I, [_P, _P]),
    'wbg_ws_replicas': (_I, [_P, _I, _P, _I, _P, _I, ctypes.POINTER(Lattice), ctypes.c_double, _I, _P, _P, _P]),
    'wbg_berry_tabulate': (_I, [_P, _P, _I, _I, _I, _I, _I, _I, ctypes.c_double, _I, _I, _P, _I, _P]),
    'wbg_berry_scan': (_I, [_P, _P, _I, _I, _I, _I, _I, ctypes.POINTER(Scan), _I, _I, _P, _I, _P]),
    'wbg_berry_omega': (_I, [_P, _P, _I, _I, _I, _I, _I, _I, ctypes.POINTER(Scan), _I, _I, _P, _I, _P]),
    'wbg_berry_morb': (_I, [_P, _P, _I, _I, _I, _I, _I, _I, _I, _I, ctypes.POINTER(Scan), _I, _I, _P, _I, _P]),
    'wbg_berry_deromega': (_I, [_P, _P, _I, _I, _I, _I, _I, _I, _I, _I, _I, ctypes.POINTER(Scan), _I, _I, _P, _I,
                                _P]),
    'wbg_kubo_workspace_size': (_I, [_I, _I, _I, ctypes.POINTER(_SZ)]),
    'wbg_kubo': (_I, [_P, _P, _I, _I, _I, _I, _I, _I, ctypes.POINTER(KuboParams), _P, _P, _P, _SZ, _P, _I, _P]),
    'wbg_dynamic_ncomp': (_I, [_I]),
    'wbg_dynamic_workspace_size': (_I, [_I, _I, _I, _I, ctypes.POINTER(_SZ)]),
    'wbg_dynamic': (_I, [_P, _P, _I, ctypes.POINTER(DynamicSpec), _I, _I, ctypes.POINTER(KuboParams), _P, _P, _P, _SZ,
                         _P, _I, _P]),
    'wbg_berry_shc': (_I, [_P, _P, _I, ctypes.POINTER(DynamicSpec), _I, _I, ctypes.POINTER(Scan), _P, _I, _P]),
    'wbg_berry_product': (_I, [_P, _P, _I, ctypes.POINTER(ProductSpec), _I, _I, ctypes.POINTER(Scan), _I, _P, _I,
                               _P]),
    'wbg_product_values': (_I, [_P, _P, _I, ctypes.POINTER(ProductSpec), _I, _I, ctypes.c_double, _P, _P, _I, _P]),
    'wbg_scan_finalize': (_I, [_P, _I, _I, ctypes.c_double, _P, _P]),
    'wbg_tetra_select': (_I, [_P, _P, _P, _P, _I, ctypes.POINTER(TetraGrid), _I, ctypes.c_double, ctypes.c_double,
                              ctypes.c_double, _I, _P, _P]),
    'wbg_band_values': (_I, [_P, _P, _I, ctypes.POINTER(FieldIndex), _I, _I, _I, _I, _I, ctypes.c_double, _P, _P, _I,
                             _P]),
    'wbg_tetra_accumulate': (_I, [_P, _P, _P, _P, _I, ctypes.POINTER(TetraGrid), _I, _P, _P, _I, _P, _I, _I, _I, _I,
                                  _P, _P]),
    'wbg_probe_fma': (_I, [_I, _I, _I, _I, _P, ctypes.POINTER(ctypes.c_double), _P]),
    'wbg_tune_candidates': (_I, [_I, _I, _I, ctypes.POINTER(_I), _I, ctypes.POINTER(_I)]),
    'wbg_tune_set': (_I, [_I, _I, _I, _I]),
    'wbg_tune_get': (_I, [_I, _I, _I, ctypes.POINTER(_I)]),
}

_lib = None


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Load libwbgpu.so; build it first if it is missing (needs nvcc)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libwbgpu.so not built at {path}")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, what):
    if status == STATUS_OK:
        return
    msg = load().wbg_status_string(status).decode()
    if status == 3:
        msg += ": " + load().wbg_last_cuda_error_string().decode()
    if status in (1, 2, 5):
        raise ValueError(f"{what}: {msg} (status {status})")
    raise RuntimeError(f"{what}: {msg} (status {status})")
