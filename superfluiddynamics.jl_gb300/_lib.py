"""ctypes binding of libgpss.so (declarations in include/gpss.h).

The library is built in place by ``build.py``; nothing here falls back to a
CPU implementation: if the shared library is missing or fails to load, every
entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgpss.so")
HEADER = os.path.join(HERE, "..", "include", "gpss.h")

GPSS_OK = 0
GPSS_EINVAL = -1
GPSS_ENOMEM = -2
GPSS_ECUDA = -3
GPSS_ENONFINITE = -4
GPSS_ETIMEOUT = -5
GPSS_ESTATE = -6
GPSS_EIO = -7
GPSS_FP64 = 64
GPSS_FP32 = 32
GPSS_FLAG_PLAIN = 1
GPSS_FLAG_NOMERGE = 2
GPSS_FLAG_NOMASSLOCK = 4
GPSS_FLAG_PIPE = 8
GPSS_FLAG_ENERGY_CACHE = 16
GPSS_FLAG_COMPENSATED = 32
GPSS_LIE = 1
GPSS_STRANG = 2

_CODES = {GPSS_EINVAL: "EINVAL", GPSS_ENOMEM: "ENOMEM", GPSS_ECUDA: "ECUDA",
          GPSS_ENONFINITE: "ENONFINITE", GPSS_ETIMEOUT: "ETIMEOUT", GPSS_ESTATE: "ESTATE",
          GPSS_EIO: "EIO"}


class GPSSError(RuntimeError):
    """Raised when a libgpss entry point returns a negative status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"gpss {_CODES.get(code, code)}: {msg}")
        self.code = code


class Diag(ctypes.Structure):
    _fields_ = [("mass", ctypes.c_double), ("energy", ctypes.c_double * 5), ("steps", ctypes.c_int64)]


_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p

# name -> (restype, argtypes); must cover every function declared in gpss.h
SIGNATURES = {
    "gpss_version": (ctypes.c_char_p, []),
    "gpss_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, _i64p, _f64p, _f64p,
                                   ctypes.c_int, ctypes.c_int]),
    "gpss_destroy": (None, [_vp]),
    "gpss_last_error": (ctypes.c_char_p, [_vp]),
    "gpss_set_params": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    "gpss_set_potential": (ctypes.c_int, [_vp, _f64p]),
    "gpss_upload": (ctypes.c_int, [_vp, _f64p]),
    "gpss_download": (ctypes.c_int, [_vp, _f64p]),
    "gpss_step": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                 ctypes.POINTER(Diag)]),
    "gpss_rk_step": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
    "gpss_implicit_step": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                          ctypes.POINTER(ctypes.c_int64)]),
    "gpss_energy": (ctypes.c_int, [_vp, _f64p]),
    "gpss_mass": (ctypes.c_int, [_vp, _f64p]),
    "gpss_norm": (ctypes.c_int, [_vp, _f64p]),
    "gpss_normalize": (ctypes.c_int, [_vp]),
    "gpss_ground_state": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_int64,
                                         ctypes.c_int, _f64p, _i64p]),
    "gpss_adjoint": (ctypes.c_int, [_vp, _f64p, ctypes.c_int, ctypes.c_int, ctypes.c_double, _f64p, _f64p,
                                    _f64p]),
    "gpss_write_h5": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "gpss_read_h5": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "gpss_h5_write_field": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _i64p, _f64p]),
    "gpss_h5_read_field": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _i64p, _f64p]),
    "gpss_h5_read_dataset": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), _i64p,
                                            _f64p, ctypes.c_int64]),
    "gpss_batch_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, _i64p, _f64p, _f64p, ctypes.c_double]),
    "gpss_batch_destroy": (None, [_vp]),
    "gpss_batch_last_error": (ctypes.c_char_p, [_vp]),
    "gpss_batch_set_run": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, _f64p, _f64p]),
    "gpss_batch_step": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, _f64p]),
    "gpss_batch_download": (ctypes.c_int, [_vp, ctypes.c_int, _f64p]),
    "gpss_batch_set_tuning": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "gpss_batch_tuning": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)]),
    "gpss_sync": (ctypes.c_int, [_vp]),
    "gpss_flush": (ctypes.c_int, [_vp]),
    "gpss_event_record": (ctypes.c_int, [_vp, ctypes.c_int]),
    "gpss_event_elapsed": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_float)]),
    "gpss_launch_count": (ctypes.c_int64, [_vp]),
    "gpss_time_pass": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, _f64p]),
    "gpss_select_device": (ctypes.c_int, [ctypes.c_int]),
    "gpss_device_count": (ctypes.c_int, []),
    "gpss_host_alloc": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int64]),
    "gpss_measure_fma_rate": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "gpss_host_free": (ctypes.c_int, [_vp]),
    "gpss_device_bytes": (ctypes.c_int64, [_vp]),
    "gpss_energy_noalloc": (ctypes.c_int, [ctypes.c_int, _i64p, _f64p, _f64p, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, _vp, _vp, _vp, _f64p]),
}

_lib = None


def header_functions(path: str = HEADER):
    """Names of the functions declared in include/gpss.h."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gpss_[a-z_0-9]+)\s*\(", text)))


def lib():
    """Load libgpss.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libgpss.so not found at {LIB_PATH}; run build.py (or "
                               "__graft_entry__.build()) first")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int, ctx=None):
    if rc != GPSS_OK:
        msg = lib().gpss_last_error(ctx)
        raise GPSSError(rc, msg.decode() if msg else "")
    return rc
