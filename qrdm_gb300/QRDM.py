"""Python module ``QRDM`` of mdessole/qrdm, on the GPU.

Same functions, positional arguments and return values as the reference's
CPython extension (QRDM_wrapper.c:131-139): ``init``, ``QRF``, ``QP3``,
``QRDM`` and ``DORMQR``.  Arrays are NumPy arrays whose raw buffers are
handed to the C ABI (libqrdm_gb300.so) exactly as the reference hands
``PyArrayObject->data`` to its C code (QRDM_wrapper.c:155-159): the memory of
``A`` is read as a column-major matrix with leading dimension ``lda``.
Unlike the reference, dtypes and buffer sizes are checked (TypeError /
ValueError) instead of silently reading foreign memory.

    import numpy as np
    from qrdm_gb300 import QRDM
    A = np.asfortranarray(X)               # m x n, float64
    jpvt = np.zeros(n, np.int32); tau = np.zeros(n); ncols = np.zeros(n, np.int32)
    info = QRDM.QRDM(102, m, n, A, m, jpvt, tau, ncols, np.array([0.9, 0.15]), 64)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import lib

_pd = C.POINTER(C.c_double)
_pi = C.POINTER(C.c_int)


def _buf(a, dtype, min_elems, name):
    if not isinstance(a, np.ndarray):
        raise TypeError(f"{name} must be a numpy array")
    if a.dtype != dtype:
        raise TypeError(f"{name} must have dtype {np.dtype(dtype).name}, got {a.dtype}")
    if not (a.flags.c_contiguous or a.flags.f_contiguous):
        raise ValueError(f"{name} must be contiguous")
    if a.size < min_elems:
        raise ValueError(f"{name} has {a.size} elements, needs {min_elems}")
    return a.ctypes.data_as(_pd if dtype == np.float64 else _pi)


def init():
    """Reference: QRDM_wrapper.c:9-13 (numpy C-API import); nothing to do."""
    return None


def QRDM(matrix_layout, m, n, A, lda, jpvt, tau, ncols, thres, DM_procedure):
    """DM-QR in place; returns info.  Reference QRDM_wrapper.c:71-100 ->
    dgeqrdm (include/QRDM.h:19-22).  The last argument is the block size nb."""
    m, n, lda, nb = int(m), int(n), int(lda), int(DM_procedure)
    pa = _buf(A, np.float64, lda * (n - 1) + m if n > 0 and m > 0 else 0, "A")
    pj = _buf(jpvt, np.int32, n, "jpvt")
    pt = _buf(tau, np.float64, min(m, n), "tau")
    pn = _buf(ncols, np.int32, max(n, 1), "ncols")
    th = _buf(thres, np.float64, 2, "thres")
    return int(lib().dgeqrdm(int(matrix_layout), m, n, pa, lda, pj, pt, pn, th, nb))


def QP3(matrix_layout, m, n, A, lda, jpvt, tau):
    """QR with column pivoting (LAPACK dgeqp3 semantics); returns info.
    Reference QRDM_wrapper.c:15-40 (LAPACKE_dgeqp3)."""
    m, n, lda = int(m), int(n), int(lda)
    pa = _buf(A, np.float64, lda * (n - 1) + m if n > 0 and m > 0 else 0, "A")
    pj = _buf(jpvt, np.int32, n, "jpvt")
    pt = _buf(tau, np.float64, min(m, n), "tau")
    return int(lib().dgeqp3(int(matrix_layout), m, n, pa, lda, pj, pt))


def QRF(matrix_layout, m, n, A, lda, tau):
    """Unpivoted Householder QR; returns info.  Reference QRDM_wrapper.c:44-66
    (LAPACKE_dgeqrf)."""
    m, n, lda = int(m), int(n), int(lda)
    pa = _buf(A, np.float64, lda * (n - 1) + m if n > 0 and m > 0 else 0, "A")
    pt = _buf(tau, np.float64, min(m, n), "tau")
    return int(lib().qrdm_dgeqrf(int(matrix_layout), m, n, pa, lda, pt))


def DORMQR(matrix_layout, m, n, k, A, lda, tau, C_, ldc):
    """C <- Q C with Q = H(1)...H(k) from A/tau (side 'L', trans 'N'); returns
    info.  Reference QRDM_wrapper.c:104-126 (LAPACKE_dormqr)."""
    m, n, k, lda, ldc = int(m), int(n), int(k), int(lda), int(ldc)
    pa = _buf(A, np.float64, lda * (k - 1) + m if k > 0 else 0, "A")
    pt = _buf(tau, np.float64, k, "tau")
    pc = _buf(C_, np.float64, ldc * (n - 1) + m if n > 0 and m > 0 else 0, "C")
    return int(lib().qrdm_dormqr(int(matrix_layout), m, n, k, pa, lda, pt, pc, ldc))
