"""ctypes binding of libqrdm_gb300.so (the C ABI in include/qrdm_gb300.h).

There is no CPU fallback: if the library is missing this module raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqrdm_gb300.so")

_pd = C.POINTER(C.c_double)
_pi = C.POINTER(C.c_int)


class Options(C.Structure):
    """struct qrdm_options."""
    _fields_ = [("precision", C.c_int), ("kstop", C.c_int), ("nancheck", C.c_int),
                ("slices", C.c_int), ("gram_margin", C.c_double),
                ("wait_limit", C.c_int), ("reserved", C.c_int * 7)]


class Stats(C.Structure):
    """struct qrdm_stats."""
    _fields_ = [("nblocks", C.c_int), ("recomputes", C.c_int), ("rechecks", C.c_int),
                ("columns", C.c_int), ("launches", C.c_int), ("timing", C.c_int),
                ("ms_total", C.c_double), ("ms_select", C.c_double), ("ms_panel", C.c_double),
                ("ms_tfactor", C.c_double), ("ms_trail", C.c_double), ("ms_norm", C.c_double),
                ("trail_flops", C.c_double), ("reserved", C.c_double * 5)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k not in ("reserved",)}


# (name, restype, argtypes) of every exported entry point
SIGNATURES = {
    "dgeqrdm": (C.c_int, [C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pi, _pd, _pi, _pd, C.c_int]),
    "dgeqrdm_ex": (C.c_int, [C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pi, _pd, _pi, _pd, C.c_int,
                             C.POINTER(Options), C.POINTER(Stats)]),
    "dgeqrdm_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                              C.c_void_p, _pi, _pd, C.c_int, C.POINTER(Options),
                              C.POINTER(Stats)]),
    "dgeqrdm_dev_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                      C.c_void_p, C.c_void_p, _pi, _pd, C.c_int, C.c_void_p]),
    "dgeqrdm_batched_dev": (C.c_int, [C.c_int, _pi, _pi, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, _pd, C.c_int, C.c_int, C.c_int]),
    "qrdm_batched_phase_cycles": (C.c_int, [C.POINTER(C.c_ulonglong), C.c_int]),
    "qrdm_panel_phase_cycles": (C.c_int, [C.POINTER(C.c_ulonglong), C.c_int]),
    "qrdm_fp64_rates": (C.c_int, [_pd, C.c_int]),
    "qrdm_legacy_mma_rates": (C.c_int, [_pd, C.c_int]),
    "qrdm_apply_jpvt_dev": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_int]),
    "qrdm_norm_diff_dev": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                     _pd]),
    "dgeqp3": (C.c_int, [C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pi, _pd]),
    "dgeqp3_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                             C.c_void_p]),
    "qrdm_dgeqrf": (C.c_int, [C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pd]),
    "qrdm_dormqr": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pd, _pd,
                              C.c_int]),
    "qrdm_dgeqrf_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p]),
    "qrdm_dormqr_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                  C.c_void_p, C.c_void_p, C.c_int]),
    "qrdm_default_options": (None, [C.POINTER(Options)]),
    "qrdm_set_stream": (C.c_int, [C.c_void_p]),
    "qrdm_version": (C.c_char_p, []),
    "qrdm_release_workspace": (C.c_int, []),
}

_LIB = None


def lib():
    """Load libqrdm_gb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def default_options(**kw) -> Options:
    o = Options()
    lib().qrdm_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o
