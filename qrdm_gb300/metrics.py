"""Accuracy measures of a (pivoted) QR factorisation, on the host (NumPy +
LAPACK dorgqr through scipy), following auxil.checkQR (auxil.py:20-105) but
normalised by ||A||_F:

    backward  = ||A[:, p] - Q R||_F / ||A||_F
    orth      = ||I - Q^T Q||_F
    rdiag     = |R_kk| profile

Q is formed from the k stored reflectors (k = factored columns); R is the
upper trapezoid of the first k rows plus the trailing block A(k:, k:) that
the factorisation left un-triangularised (checkQR's R_22).
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import lapack


def form_q(Aout: np.ndarray, tau: np.ndarray, k: int) -> np.ndarray:
    """m x m orthogonal Q = H(1)...H(k) (m x min(m, n) when k == min(m, n))."""
    m, n = Aout.shape
    full = k < min(m, n) or m <= n
    cols = m if full else n
    a = np.zeros((m, cols), order="F")
    kk = min(k, cols)
    a[:, :kk] = Aout[:, :kk]
    q, _, info = lapack.dorgqr(a, np.asarray(tau[:kk], dtype=np.float64), lwork=max(1, 64 * cols))
    if info != 0:
        raise RuntimeError(f"dorgqr info={info}")
    return q


def r_factor(Aout: np.ndarray, k: int, rows: int) -> np.ndarray:
    m, n = Aout.shape
    R = np.zeros((rows, n))
    R[:k, :] = np.triu(Aout[:k, :])
    if k < rows:
        R[k:, k:] = Aout[k:rows, k:]
    return R


def factor_metrics(A0: np.ndarray, Aout: np.ndarray, tau: np.ndarray, jpvt: np.ndarray,
                   k: int | None = None) -> dict:
    m, n = A0.shape
    mn = min(m, n)
    k = mn if k is None else min(int(k), mn)
    q = form_q(Aout, tau, k)
    R = r_factor(Aout, k, q.shape[1])
    p = np.asarray(jpvt) - 1
    anorm = np.linalg.norm(A0)
    be = np.linalg.norm(A0[:, p] - q @ R) / (anorm if anorm > 0 else 1.0)
    orth = np.linalg.norm(np.eye(q.shape[1]) - q.T @ q)
    return {"backward": float(be), "orth": float(orth),
            "rdiag": np.abs(np.diag(Aout[:k, :k])).copy(), "k": k}
