"""qrdm_gb300 -- QR with Deviation Maximization pivoting on one NVIDIA GB300.

GPU drop-in for mdessole/qrdm: the C ABI (include/qrdm_gb300.h, built into
libqrdm_gb300.so from csrc/) and the ``QRDM`` Python module
(``from qrdm_gb300 import QRDM``).  This package adds NumPy/torch
conveniences on top of the same entry points:

    res = qrdm_gb300.dgeqrdm(A, nb=64, delta=0.9, tau_=0.15)
    res["A"], res["jpvt"], res["tau"], res["ncols"], res["info"]
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Options, Stats, default_options, lib

PREC = {"fp64": 0, "mixed": 1}


def dgeqrdm(A0, nb: int = 64, delta: float = 0.9, tau_: float = 0.15, stop: int = 0,
            eta: float | None = None, precision: str = "fp64", kstop: int = 0, jpvt=None,
            nancheck: bool = True) -> dict:
    """Factor a copy of the host matrix A0 (m x n) with DM-QR on the GPU.
    Returns dict(A, jpvt, tau, ncols, info, stats)."""
    A = np.array(A0, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    jp = np.zeros(n, np.int32) if jpvt is None else np.array(jpvt, np.int32)
    tau = np.zeros(min(m, n), np.float64)
    ncols = np.zeros(n, np.int32)
    ncols[0] = stop
    thres = np.array([delta, tau_, 0.0 if eta is None else eta], np.float64)
    opt = default_options(precision=PREC[precision], kstop=int(kstop), nancheck=int(nancheck))
    st = Stats()
    pd, pi = C.POINTER(C.c_double), C.POINTER(C.c_int)
    info = lib().dgeqrdm_ex(102, m, n, A.ctypes.data_as(pd), m, jp.ctypes.data_as(pi),
                            tau.ctypes.data_as(pd), ncols.ctypes.data_as(pi),
                            thres.ctypes.data_as(pd), int(nb), C.byref(opt), C.byref(st))
    return {"A": A, "jpvt": jp, "tau": tau, "ncols": ncols, "info": int(info),
            "stats": st.as_dict()}


def dgeqrdm_device(a, jpvt, tau, nb: int = 64, delta: float = 0.9, tau_: float = 0.15,
                   stop: int = 0, eta: float | None = None, precision: str = "fp64",
                   kstop: int = 0, nancheck: bool = True, ncols=None) -> dict:
    """DM-QR on device-resident torch tensors, in place.  ``a`` is a CUDA
    float64 tensor holding the matrix column-major (e.g. ``X.t().contiguous()``
    of a row-major m x n X has shape (n, m)); pass m, n via ``a.shape[::-1]``.
    jpvt: int32 CUDA tensor (n), tau: float64 CUDA tensor (min(m, n))."""
    n, m = a.shape
    nc = np.zeros(n, np.int32) if ncols is None else ncols
    nc[0] = stop
    thres = np.array([delta, tau_, 0.0 if eta is None else eta], np.float64)
    opt = default_options(precision=PREC[precision], kstop=int(kstop), nancheck=int(nancheck))
    st = Stats()
    info = lib().dgeqrdm_dev(102, m, n, C.c_void_p(a.data_ptr()), m, C.c_void_p(jpvt.data_ptr()),
                             C.c_void_p(tau.data_ptr()),
                             nc.ctypes.data_as(C.POINTER(C.c_int)),
                             thres.ctypes.data_as(C.POINTER(C.c_double)), int(nb), C.byref(opt),
                             C.byref(st))
    return {"ncols": nc, "info": int(info), "stats": st.as_dict()}


__all__ = ["dgeqrdm", "dgeqrdm_device", "Options", "Stats", "default_options", "lib", "PREC"]
