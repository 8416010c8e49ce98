"""Rank-revealing helpers over the GPU factorisation, with the names,
arguments and array conventions of the reference's ``auxil`` module
(auxil.py:6-200), so code written against ``auxil`` + ``QRDM`` runs on this
package by swapping the imports.

Array convention (the reference's, for matrix_layout = 102): a column-major
m x n matrix is held in a C-ordered NumPy array of shape (n, m), i.e. the
NumPy transpose; ``getR``/``checkQR``/``low_rank`` return ordinary (m x ...)
NumPy matrices.  Q is applied with this package's GPU DORMQR.  Layout 101 is
rejected, as in the rest of the package.
"""
from __future__ import annotations

import numpy as np

from . import QRDM


def rank_from_sv(s, tol: float = 5.0e-9) -> int:
    """Numerical rank read off singular values or |diag(R)| of an RRQR, in
    the reference's convention (auxil.py:6-17): the 1-based position of the
    first value whose magnitude is below tol (values need not be sorted),
    or len(s) if there is none."""
    small = np.flatnonzero(np.abs(np.asarray(s)) < tol)
    return int(small.min()) + 1 if small.size else int(len(s))


def _order(m, n, k):
    mn = min(m, n)
    return mn if (k == 0 or k > mn) else int(k)


def getR(matrix_layout, m, n, A, k=0):
    """R factor (m x n) of a factorisation stored in A (auxil.py:107-154):
    the upper triangle of the first k columns' rows and, for k < n, the
    remaining block untouched (R_12 above R_22)."""
    if matrix_layout != 102:
        raise ValueError("only matrix_layout = 102 (column-major) is supported")
    k = _order(m, n, k)
    At = np.asarray(A).T  # m x n view of the column-major factor
    if k == n:
        return np.triu(At)
    R = np.zeros_like(At)
    R[:, :k] = np.triu(At[:, :k])
    R[:, k:] = At[:, k:]
    return R


def checkQR(matrix_layout, m, n, A, M, tau, jpvt, k=0, check_err=True, verbose=False):
    """(Q, R, err, errQ) as auxil.checkQR (auxil.py:20-105): Q (m x m) from
    the k stored reflectors, R from getR, err = ||M[:, p] - Q R||_F and
    errQ = ||I - Q^T Q||_F (absolute), M the original matrix in the same
    (n, m) convention as A."""
    if matrix_layout != 102:
        raise ValueError("only matrix_layout = 102 (column-major) is supported")
    k = _order(m, n, k)
    Qt = np.ascontiguousarray(np.eye(m))  # column-major m x m (symmetric start)
    # all m columns of Q (auxil.checkQR forms min(m, n) of them into an
    # identity, which leaves the others unorthogonalised when m > n)
    info = QRDM.DORMQR(102, m, m, k, np.ascontiguousarray(A), m, np.asarray(tau, np.float64), Qt, m)
    if info != 0:
        raise RuntimeError(f"DORMQR info={info}")
    Q = Qt.T  # back to an ordinary m x m matrix
    R = getR(102, m, n, A, k)
    err = errQ = 0.0
    if check_err:
        errQ = float(np.linalg.norm(np.eye(m) - Q.T @ Q))
        p = np.asarray(jpvt) - 1
        err = float(np.linalg.norm(np.asarray(M).T[:, p] - Q @ R))
        if verbose:
            print("||Q.T*Q - I|| =", errQ)
            print("||A[:,p] - Q*R|| =", err)
    return Q, R, err, errQ


def low_rank(matrix_layout, m, n, M, A, tau, jpvt, k):
    """Rank-k approximation Q [R_11 R_12; 0 0] of the pivoted matrix
    (auxil.py:156-200), M the factorisation in the (n, m) convention; the
    result is an ordinary m x n matrix (columns in pivoted order)."""
    if matrix_layout != 102:
        raise ValueError("only matrix_layout = 102 (column-major) is supported")
    k = _order(m, n, k)
    Mt = np.asarray(M).T  # m x n factor
    top = np.zeros((m, n))
    top[:k, :] = np.triu(Mt[:k, :])
    C = np.ascontiguousarray(top.T)  # column-major m x n in the (n, m) convention
    info = QRDM.DORMQR(102, m, n, k, np.ascontiguousarray(M), m, np.asarray(tau, np.float64), C, m)
    if info != 0:
        raise RuntimeError(f"DORMQR info={info}")
    return C.T


# ------------------------------------------------------------ on the device
# The same helpers on device-resident torch tensors (float64 CUDA tensors in
# the (n, m) convention above, jpvt an int32 CUDA tensor): Q is formed and
# applied with the library's DORMQR, A P with its column gather
# (qrdm_apply_jpvt_dev), the Frobenius norms with its device reduction
# (qrdm_norm_diff_dev); only Q^T Q, which auxil.checkQR forms explicitly,
# uses a library GEMM (torch.matmul).  Nothing leaves the device but the two
# norms.

def _lib():
    from ._lib import lib

    return lib()


def _ptr(t):
    import ctypes as C

    return C.c_void_p(t.data_ptr())


def _check_dev(t, name, dtype=None):
    import torch

    if not isinstance(t, torch.Tensor) or not t.is_cuda or not t.is_contiguous():
        raise ValueError(f"{name} must be a contiguous CUDA tensor")
    if dtype is not None and t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}")


def getR_dev(matrix_layout, m, n, A, k=0):
    """getR on the device: R of the factorisation in the (n, m) CUDA tensor
    A, returned in the same (n, m) convention."""
    import torch

    if matrix_layout != 102:
        raise ValueError("only matrix_layout = 102 (column-major) is supported")
    _check_dev(A, "A", torch.float64)
    k = _order(m, n, k)
    At = A.T  # m x n view
    R = torch.zeros((n, m), dtype=torch.float64, device=A.device)
    Rt = R.T
    Rt[:, :k] = torch.triu(At[:, :k])
    if k < n:
        Rt[:, k:] = At[:, k:]
    return R


def _on_torch_stream():
    """Run the library on torch's current stream (ordered with the tensors'
    producers)."""
    import ctypes as C

    import torch

    _lib().qrdm_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))


def _dormqr_dev(m, ncol, k, A, tau, Cm):
    _on_torch_stream()
    info = _lib().qrdm_dormqr_dev(102, m, ncol, k, _ptr(A), m, _ptr(tau), _ptr(Cm), m)
    if info != 0:
        raise RuntimeError(f"qrdm_dormqr_dev info={info}")


def _norm_diff(m, n, X, Y=None):
    import ctypes as C

    out = C.c_double(0.0)
    _on_torch_stream()
    r = _lib().qrdm_norm_diff_dev(m, n, _ptr(X), m, _ptr(Y) if Y is not None else None, m, C.byref(out))
    if r != 0:
        raise RuntimeError(f"qrdm_norm_diff_dev returned {r}")
    return float(out.value)


def apply_jpvt_dev(m, n, M, jpvt):
    """A P on the device: column j of the result is column jpvt[j] - 1 of
    the (n, m) CUDA tensor M; returned in the same convention."""
    import torch

    _check_dev(M, "M", torch.float64)
    _check_dev(jpvt, "jpvt", torch.int32)
    out = torch.empty_like(M)
    _on_torch_stream()
    r = _lib().qrdm_apply_jpvt_dev(m, n, _ptr(M), m, _ptr(jpvt), _ptr(out), m)
    if r != 0:
        raise RuntimeError(f"qrdm_apply_jpvt_dev returned {r}")
    return out


def checkQR_dev(matrix_layout, m, n, A, M, tau, jpvt, k=0, check_err=True):
    """checkQR on the device: (Q, R, err, errQ) with Q the m x m orthogonal
    factor as an (m, m) CUDA tensor holding Q column-major (Q^T row-major),
    R as getR_dev, err = ||M[:, p] - Q R||_F (Q R formed by DORMQR applied to
    R, M[:, p] by the column gather) and errQ = ||I - Q^T Q||_F, both
    absolute, as auxil.checkQR."""
    import torch

    if matrix_layout != 102:
        raise ValueError("only matrix_layout = 102 (column-major) is supported")
    for t, nm in ((A, "A"), (M, "M"), (tau, "tau")):
        _check_dev(t, nm, torch.float64)
    _check_dev(jpvt, "jpvt", torch.int32)
    k = _order(m, n, k)
    Qt = torch.eye(m, dtype=torch.float64, device=A.device)  # column-major identity
    _dormqr_dev(m, m, k, A, tau, Qt)
    R = getR_dev(102, m, n, A, k)
    err = errQ = 0.0
    if check_err:
        QR = R.clone()
        _dormqr_dev(m, n, k, A, tau, QR)
        AP = apply_jpvt_dev(m, n, M, jpvt)
        err = _norm_diff(m, n, AP, QR)
        QtQ = Qt @ Qt.T  # rows of Qt are the columns of Q: (Q^T Q) in column-major order
        eye = torch.eye(m, dtype=torch.float64, device=A.device)
        errQ = _norm_diff(m, m, eye, QtQ.contiguous())
    return Qt, R, err, errQ


def low_rank_dev(matrix_layout, m, n, M, A, tau, jpvt, k):
    """low_rank on the device: Q [R_11 R_12; 0 0] from the factorisation in
    the (n, m) CUDA tensor M, returned as an m x n view (columns in pivoted
    order), as auxil.low_rank."""
    import torch

    if matrix_layout != 102:
        raise ValueError("only matrix_layout = 102 (column-major) is supported")
    _check_dev(M, "M", torch.float64)
    _check_dev(tau, "tau", torch.float64)
    k = _order(m, n, k)
    top = torch.zeros((n, m), dtype=torch.float64, device=M.device)
    top.T[:k, :] = torch.triu(M.T[:k, :])
    _dormqr_dev(m, n, k, M, tau, top)
    return top.T
