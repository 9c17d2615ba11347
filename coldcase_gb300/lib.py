"""ctypes binding of libcovgpu.so (the C ABI declared in include/covgpu.h).

There is no fallback: if the library is missing or no sm_103 device is
present, every call raises CovError.
"""
import ctypes
import os
import re

import numpy as np

from . import _build

COV_OK = 0
ERRORS = {
    -1: "COV_EINVAL: bad parameter or outside the domain",
    -2: "COV_ENOMEM: device allocation failed",
    -3: "COV_ESTATE: call out of order",
    -4: "COV_ETIMEOUT: a bounded device-side wait or a launch budget ran out",
    -5: "COV_EDRIFT: an in-kernel invariant check failed",
    -6: "COV_ENODEV: no usable sm_103 device",
    -7: "COV_ERANGE: request exceeds a fixed capacity",
}


class CovError(RuntimeError):
    def __init__(self, rc, what=""):
        self.rc = rc
        if rc <= -100:
            msg = "CUDA runtime error %d" % (-rc - 100)
        else:
            msg = ERRORS.get(rc, "error %d" % rc)
        super().__init__("%s: %s" % (what, msg) if what else msg)


class CovMoveRec(ctypes.Structure):
    _fields_ = [("it", ctypes.c_int64), ("u", ctypes.c_int64), ("delta", ctypes.c_int64),
                ("unc", ctypes.c_int64), ("unc_end", ctypes.c_int64), ("best", ctypes.c_int64),
                ("ncand", ctypes.c_int32), ("ncw", ctypes.c_int32), ("i", ctypes.c_int32),
                ("p", ctypes.c_int32), ("v", ctypes.c_int32), ("kicked", ctypes.c_int32)]


MOVE_DTYPE = np.dtype([("it", "<i8"), ("u", "<i8"), ("delta", "<i8"), ("unc", "<i8"),
                       ("unc_end", "<i8"), ("best", "<i8"), ("ncand", "<i4"), ("ncw", "<i4"),
                       ("i", "<i4"), ("p", "<i4"), ("v", "<i4"), ("kicked", "<i4")])
assert MOVE_DTYPE.itemsize == ctypes.sizeof(CovMoveRec) == 72


class CovParams(ctypes.Structure):
    _fields_ = [("q", ctypes.c_int32), ("n", ctypes.c_int32), ("R", ctypes.c_int32),
                ("M", ctypes.c_int32), ("seed", ctypes.c_uint64), ("tabu", ctypes.c_int32),
                ("kick", ctypes.c_int32), ("cand", ctypes.c_int32), ("trace", ctypes.c_int32),
                ("stall", ctypes.c_int64), ("trace_cap", ctypes.c_int64), ("wide", ctypes.c_int32),
                ("fix0", ctypes.c_int32), ("sa", ctypes.c_int32), ("noise", ctypes.c_int32),
                ("t0", ctypes.c_double), ("cool", ctypes.c_double), ("tmin", ctypes.c_double)]


class CovStatus(ctypes.Structure):
    _fields_ = [("it", ctypes.c_int64), ("uncovered", ctypes.c_int64), ("best", ctypes.c_int64),
                ("kicks", ctypes.c_int64), ("trace_n", ctypes.c_int64), ("status", ctypes.c_int32),
                ("finished", ctypes.c_int32), ("ul_valid", ctypes.c_int32), ("ul_n", ctypes.c_int32)]


class CovSymParams(ctypes.Structure):
    _fields_ = [("q", ctypes.c_int32), ("n", ctypes.c_int32), ("R", ctypes.c_int32), ("M", ctypes.c_int32),
                ("orbits", ctypes.c_int32), ("kick", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("stall", ctypes.c_int64), ("cand", ctypes.c_int32), ("trace", ctypes.c_int32),
                ("trace_cap", ctypes.c_int64)]


_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_PI32 = ctypes.POINTER(ctypes.c_int32)
_PI64 = ctypes.POINTER(ctypes.c_int64)
_PU8 = ctypes.POINTER(ctypes.c_uint8)
_PU32 = ctypes.POINTER(ctypes.c_uint32)

SIGNATURES = {
    "cov_pool_create": (ctypes.c_int, [_I32, _I32, ctypes.POINTER(_P)]),
    "cov_pool_set_budget": (ctypes.c_int, [_P, ctypes.c_double]),
    "cov_pool_set_param": (ctypes.c_int, [_P, ctypes.c_char_p, _I64]),
    "cov_pool_set_slot_param": (ctypes.c_int, [_P, _I32, ctypes.c_char_p, _I64]),
    "cov_slot_bytes": (ctypes.c_size_t, [ctypes.POINTER(CovParams)]),
    "cov_device_memory": (ctypes.c_int, [_PI64, _PI64]),
    "cov_pool_add": (ctypes.c_int, [_P, ctypes.POINTER(CovParams), _PU8, _I32, _I32, _PI32]),
    "cov_pool_load": (ctypes.c_int, [_P, _I32, ctypes.c_uint64, _PU8, _I32, _I32]),
    "cov_pool_run": (ctypes.c_int, [_P, _I64, _I64]),
    "cov_pool_run_async": (ctypes.c_int, [_P, _I64, _I64]),
    "cov_pool_graph_run": (ctypes.c_int, [_P, _I64, _I64, _I32]),
    "cov_pool_sync": (ctypes.c_int, [_P]),
    "cov_pool_set_stream": (ctypes.c_int, [_P, _P]),
    "cov_pool_status_all": (ctypes.c_int, [_P, ctypes.POINTER(CovStatus), _I32]),
    "cov_pool_status": (ctypes.c_int, [_P, _I32, ctypes.POINTER(CovStatus)]),
    "cov_pool_get_code": (ctypes.c_int, [_P, _I32, _PU8]),
    "cov_pool_get_best": (ctypes.c_int, [_P, _I32, _PU8]),
    "cov_pool_get_cnt": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.c_uint16)]),
    "cov_pool_get_private": (ctypes.c_int, [_P, _I32, _PI32]),
    "cov_pool_get_tabu": (ctypes.c_int, [_P, _I32, _PI32]),
    "cov_pool_get_prof": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.c_uint64)]),
    "cov_pool_get_rng": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.c_uint64)]),
    "cov_pool_get_trace": (ctypes.c_int, [_P, _I32, ctypes.POINTER(CovMoveRec), _I64, _PI64]),
    "cov_pool_resume": (ctypes.c_int, [_P, _I32]),
    "cov_pool_remove": (ctypes.c_int, [_P, _I32]),
    "cov_pool_destroy": (ctypes.c_int, [_P]),
    "cov_verify": (ctypes.c_int, [_I32, _I32, _I32, _PU8, _I32, _PI64]),
    "cov_mindist": (ctypes.c_int, [_I32, _I32, _PU8, _I32, _PU8, _PI64, _PI32]),
    "cov_count": (ctypes.c_int, [_I32, _I32, _I32, _PU8, _I32, ctypes.POINTER(ctypes.c_uint16), _PI64]),
    "cov_mindist_dev": (ctypes.c_int, [_I32, _I32, _P, _I32, _P, _P]),
    "cov_count_dev": (ctypes.c_int, [_I32, _I32, _I32, _P, _I32, _P, _P]),
    "cov_count_above_dev": (ctypes.c_int64, [_I32, _I32, _P, _I32, _P]),
    "cov_mindist_dev_static": (ctypes.c_int, [_I32, _I32, _P, _I32, _P, _P]),
    "cov_finish": (ctypes.c_int, [_I32, _I32, _I32, _I32, _PU8, _I32, _I32, _PU8, _PI32, _PI64]),
    "cov_chain_run": (ctypes.c_int, [ctypes.c_int] * 5 + [ctypes.c_longlong, ctypes.c_ulonglong, ctypes.c_int,
                                                          _PU8, _PU8, _PI32, _PI32, _PI64]),
    "cov_sym_create": (ctypes.c_int, [_I32, _I32, ctypes.POINTER(_P)]),
    "cov_sym_destroy": (ctypes.c_int, [_P]),
    "cov_sym_set_budget": (ctypes.c_int, [_P, ctypes.c_double]),
    "cov_sym_set_param": (ctypes.c_int, [_P, ctypes.c_char_p, _I64]),
    "cov_sym_orbits": (ctypes.c_int, [ctypes.POINTER(CovSymParams)]),
    "cov_sym_slot_bytes": (ctypes.c_size_t, [ctypes.POINTER(CovSymParams)]),
    "cov_sym_add": (ctypes.c_int, [_P, ctypes.POINTER(CovSymParams), _PI32]),
    "cov_sym_remove": (ctypes.c_int, [_P, _I32]),
    "cov_sym_set_slot_param": (ctypes.c_int, [_P, _I32, ctypes.c_char_p, _I64]),
    "cov_sym_run": (ctypes.c_int, [_P, _I64]),
    "cov_sym_status": (ctypes.c_int, [_P, _I32, ctypes.POINTER(CovStatus)]),
    "cov_sym_resume": (ctypes.c_int, [_P, _I32]),
    "cov_sym_get_rep": (ctypes.c_int, [_P, _I32, _PU8]),
    "cov_sym_get_best": (ctypes.c_int, [_P, _I32, _PU8]),
    "cov_sym_get_cnt": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.c_uint16)]),
    "cov_sym_get_trace": (ctypes.c_int, [_P, _I32, ctypes.POINTER(CovMoveRec), _I64, _PI64]),
    "cov_sym_get_rng": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.c_uint64)]),
    "cov_sym_get_prof": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.c_uint64)]),
    "cov_lns_create": (ctypes.c_int, [_I32, _I32, _I32, ctypes.POINTER(_P)]),
    "cov_lns_destroy": (ctypes.c_int, [_P]),
    "cov_lns_recount": (ctypes.c_int, [_P, _PU32, _I32]),
    "cov_lns_map": (ctypes.c_int, [_P, _I32]),
    "cov_lns_map_max": (ctypes.c_int, [_P, _PI32]),
    "cov_lns_map_hist": (ctypes.c_int, [_P, _I32, _I32, _PI64]),
    "cov_lns_map_extract": (ctypes.c_int, [_P, _I32, _I64, _PU32, _PI32, _PI64]),
    "cov_lns_map_read": (ctypes.c_int, [_P, _PU32, _I32, _PI32]),
    "cov_lns_ball": (ctypes.c_int, [_P, _PU32, _I32, _I32, _I32, _PI32]),
    "cov_lns_count": (ctypes.c_int, [_P, _I32, _PI64]),
    "cov_lns_apply": (ctypes.c_int, [_P, _PU32, _I32, _I32, _PI64]),
    "cov_lns_peel": (ctypes.c_int, [_P, _PU32, _I32, ctypes.POINTER(ctypes.c_uint8), _PI32, _PI64]),
    "cov_lns_greedy": (ctypes.c_int, [_P, _I32, _I64, _PU32, _PI32, _PI64, _PI64]),
    "cov_lns_uncovered": (ctypes.c_int, [_P, _I64, _PU32, _PI64]),
    "cov_lns_get_cnt": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint16)]),
    "cov_lns_get_map": (ctypes.c_int, [_P, _PI32]),
}

_lib = None


def header_symbols():
    """Names of every function include/covgpu.h declares."""
    path = os.path.join(_build.INCLUDE, "covgpu.h")
    txt = open(path).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cov\w+)\s*\(", txt)))


def load(build_if_missing=False):
    """Load libcovgpu.so (building it first when asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise CovError(-6, "libcovgpu.so is not built (run __graft_entry__.build())")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, what=""):
    if rc != COV_OK:
        raise CovError(rc, what)
    return rc


def u8ptr(a):
    return a.ctypes.data_as(_PU8)


def as_code(code, q, n):
    """Contiguous uint8 (m, n) view of a code; validates the digits."""
    a = np.ascontiguousarray(np.asarray(code, dtype=np.uint8).reshape(-1, n))
    if a.size and int(a.max()) >= q:
        raise ValueError("digit out of range for q=%d" % q)
    return a
