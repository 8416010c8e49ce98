"""``DMrrqr`` with the signature and outputs of the reference's NumPy
prototype (QR.py:324-505), computed by this package's GPU DM-QR.

    Q, R, piv, it = DMrrqr(A, kDM=2, thres=0.2222, thresnrm=0.5)

gives A[:, piv] = Q R with Q (m x m) orthogonal, R (m x n) upper
trapezoidal, piv 0-based and it the number of DM blocks.  The mapping of
parameters: kDM -> the maximum DM block size nb, thres (the cosine bound)
-> delta, thresnrm (the relative norm bound of the candidates) -> tau_.

The prototype differs from the C algorithm it preceded, and this adaptor
follows the C algorithm (src/dgeqrdm_work.c), so pivots can differ: the
prototype keeps up to 2 kDM candidates (QR.py:274-275), downdates its cosine
matrix from the previous one instead of recomputing it (QR.py:468-481),
orders candidates with an unstable argsort, and stops when the largest
squared residual norm drops below tol; the C algorithm caps the candidates at
nb, recomputes the candidates' cosines every block, orders them by (norm,
index) and factors all min(m, n) columns.
"""
from __future__ import annotations

import numpy as np


def DMrrqr(A, kDM: int = 2, thres: float = 0.2222, thresnrm: float = 0.5, inplace: bool = False,
           tol: float = 1e-17, verbose: bool = False, precision: str = "fp64"):
    from . import dgeqrdm
    from .QRDM import DORMQR

    A = np.asarray(A, dtype=np.float64)
    m, n = A.shape
    r = dgeqrdm(A, nb=int(kDM), delta=float(thres), tau_=float(thresnrm), precision=precision)
    if r["info"] != 0:
        raise RuntimeError(f"dgeqrdm info={r['info']}")
    F = r["A"]  # column-major factor (Fortran-ordered m x n)
    k = min(m, n)
    Qt = np.ascontiguousarray(np.eye(m))
    info = DORMQR(102, m, m, k, np.ascontiguousarray(F.T), m, r["tau"], Qt, m)
    if info != 0:
        raise RuntimeError(f"DORMQR info={info}")
    Q = Qt.T
    R = np.triu(F)
    piv = r["jpvt"].astype(np.int64) - 1
    it = int(np.count_nonzero(r["ncols"]))
    if verbose:
        print("blocks", it, "sizes", r["ncols"][:it])
    if inplace:
        A[...] = R
    return Q, R, piv, it
