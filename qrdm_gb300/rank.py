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
