"""ctypes front end of the CPU oracle (oracle/dmqr_oracle.c) and of the
compiled reference (oracle/_ref/libqrdm_ref.so, built by oracle/build_ref.sh).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.

Both libraries expose the reference calling convention of ``dgeqrdm``
(include/QRDM.h:19-22): column-major (layout 102) FP64 matrix with leading
dimension ``lda``, int32 ``jpvt`` (in: nonzero = fixed column; out: 1-based
permutation), ``tau``, int32 ``ncols`` (in: ncols[0] = stop mode; out: DM block
sizes), ``thres = [delta, tau_, (eta)]`` and the block size ``nb``.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD_DIR, "libdmqr_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libqrdm_ref.so")
NMARGIN = 6
MARGIN_NAMES = ("candidate", "order", "cosine", "panel_exit", "recompute", "stop")

_pd = C.POINTER(C.c_double)
_pi = C.POINTER(C.c_int)


def openblas_path() -> str:
    """Path of the OpenBLAS bundled with scipy (the oracle's BLAS/LAPACK)."""
    import numpy
    import scipy

    pats = [os.path.dirname(scipy.__file__) + ".libs/libscipy_openblas*.so*",
            os.path.dirname(numpy.__file__) + ".libs/libscipy_openblas*.so*",
            os.path.dirname(scipy.__file__) + ".libs/*openblas*.so*",
            os.path.dirname(numpy.__file__) + ".libs/*openblas*.so*"]
    for pat in pats:
        cands = sorted(glob.glob(pat))
        if cands:
            return cands[0]
    raise RuntimeError("no OpenBLAS shared object found next to scipy/numpy")


def build_oracle(force: bool = False) -> str:
    """Compile the oracle restatement with gcc (plain C, no GPU)."""
    src = os.path.join(HERE, "dmqr_oracle.c")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)):
        return ORACLE_SO
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = ORACLE_SO + f".{os.getpid()}.tmp"
    # -ffp-contract=off: no FMA contraction, so x86 and Arm hosts round alike
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                           "-o", tmp, src, "-ldl", "-lm"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_root(root: str | None = None) -> str | None:
    """Root of the reference sources: the argument, else the environment
    variable QRDM_REFERENCE_ROOT; None when neither is given."""
    return root or os.environ.get("QRDM_REFERENCE_ROOT") or None


def reference_sources_present(root: str | None = None) -> bool:
    r = reference_root(root)
    return bool(r) and os.path.isdir(os.path.join(r, "src"))


def reference_built() -> bool:
    """True once build_ref.sh has produced the compiled reference."""
    return os.path.exists(REF_SO)


def build_reference(root: str | None = None) -> str | None:
    """Compile the unmodified reference sources found under ``root`` (or
    QRDM_REFERENCE_ROOT); nothing happens where they are absent."""
    r = reference_root(root)
    if not reference_sources_present(r):
        return REF_SO if reference_built() else None
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh"), r])
    return REF_SO if reference_built() else None


def _dp(a):
    return a.ctypes.data_as(_pd)


def _ip(a):
    return a.ctypes.data_as(_pi)


def _check_args(A, jpvt, tau, ncols):
    assert A.dtype == np.float64 and A.flags.f_contiguous, "A must be float64, Fortran order"
    assert jpvt.dtype == np.int32 and ncols.dtype == np.int32
    assert tau.dtype == np.float64


class Oracle:
    """The C restatement of the reference DM-QR (plus LAPACK QP3/QRF/DORMQR)."""

    def __init__(self, threads: int | None = 1):
        lib = C.CDLL(build_oracle())
        rc = lib.oracle_init(openblas_path().encode())
        if rc != 0:
            raise RuntimeError(f"oracle_init failed ({rc})")
        lib.oracle_dgeqrdm_ex.restype = C.c_int
        lib.oracle_dgeqrdm_ex.argtypes = [C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pi, _pd,
                                          _pi, _pd, C.c_int, _pd, _pd, C.c_int, _pi]
        lib.oracle_dgeqp3.argtypes = [C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pi, _pd]
        lib.oracle_dgeqrf.argtypes = [C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pd]
        lib.oracle_dormqr.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pd,
                                      _pd, C.c_int]
        self.lib = lib
        if threads is not None:
            lib.oracle_set_threads(int(threads))

    def set_threads(self, t: int):
        self.lib.oracle_set_threads(int(t))

    def dgeqrdm(self, layout, m, n, A, lda, jpvt, tau, ncols, thres, nb,
                margins: np.ndarray | None = None, kstop: int = 0,
                block_margin: np.ndarray | None = None):
        """In-place DM-QR, reference calling convention; returns info.
        margins (6) / block_margin (n): decision margins in units of
        eps * ||A||_F (see dmqr_oracle.c)."""
        _check_args(A, jpvt, tau, ncols)
        thres = np.ascontiguousarray(thres, dtype=np.float64)
        nblk = np.zeros(1, np.int32)
        mp = _dp(margins) if margins is not None else None
        bp = _dp(block_margin) if block_margin is not None else None
        return self.lib.oracle_dgeqrdm_ex(layout, m, n, _dp(A), lda, _ip(jpvt), _dp(tau),
                                          _ip(ncols), _dp(thres), nb, mp, bp, kstop,
                                          _ip(nblk))

    def dgeqp3(self, layout, m, n, A, lda, jpvt, tau):
        return self.lib.oracle_dgeqp3(layout, m, n, _dp(A), lda, _ip(jpvt), _dp(tau))

    def dgeqrf(self, layout, m, n, A, lda, tau):
        return self.lib.oracle_dgeqrf(layout, m, n, _dp(A), lda, _dp(tau))

    def dormqr(self, layout, m, n, k, A, lda, tau, Cm, ldc):
        return self.lib.oracle_dormqr(layout, m, n, k, _dp(A), lda, _dp(tau), _dp(Cm), ldc)


class Reference:
    """The compiled, unmodified reference (only in the container that holds
    its sources; see oracle/build_ref.sh)."""

    def __init__(self):
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(REF_SO)
        lib = C.CDLL(REF_SO)
        lib.dgeqrdm.restype = C.c_int
        lib.dgeqrdm.argtypes = [C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pi, _pd, _pi, _pd,
                                C.c_int]
        lib.dgeqp3.argtypes = [C.c_int, C.c_int, C.c_int, _pd, C.c_int, _pi, _pd]
        self.lib = lib

    def dgeqrdm(self, layout, m, n, A, lda, jpvt, tau, ncols, thres, nb):
        _check_args(A, jpvt, tau, ncols)
        thres = np.ascontiguousarray(thres, dtype=np.float64)
        return self.lib.dgeqrdm(layout, m, n, _dp(A), lda, _ip(jpvt), _dp(tau), _ip(ncols),
                                _dp(thres), nb)

    def dgeqp3(self, layout, m, n, A, lda, jpvt, tau):
        return self.lib.dgeqp3(layout, m, n, _dp(A), lda, _ip(jpvt), _dp(tau))


def run_dmqr(impl, A0: np.ndarray, delta=0.9, tau_=0.15, nb=64, stop=0, eta=None,
             jpvt0=None, kstop=0, margins=False):
    """Convenience: factor a copy of A0 with ``impl`` (Oracle or Reference).
    Returns dict(A, jpvt, tau, ncols, info[, margins])."""
    A = np.array(A0, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    jpvt = np.zeros(n, np.int32) if jpvt0 is None else np.array(jpvt0, np.int32)
    tau = np.zeros(min(m, n), np.float64)
    ncols = np.zeros(n, np.int32)
    ncols[0] = stop
    thres = np.array([delta, tau_, 0.0 if eta is None else eta], np.float64)
    out = {}
    if isinstance(impl, Oracle):
        mg = np.zeros(NMARGIN, np.float64) if margins else None
        bm = np.zeros(n, np.float64) if margins else None
        info = impl.dgeqrdm(102, m, n, A, m, jpvt, tau, ncols, thres, nb, mg, kstop, bm)
        if margins:
            out["margins"] = dict(zip(MARGIN_NAMES, mg.tolist()))
            out["block_margin"] = bm
    else:
        info = impl.dgeqrdm(102, m, n, A, m, jpvt, tau, ncols, thres, nb)
    out.update(A=A, jpvt=jpvt, tau=tau, ncols=ncols, info=info)
    return out


def separated_prefix(ref: dict, gap: float) -> tuple[int, int]:
    """(blocks, columns) of the leading DM blocks whose every decision is at
    least ``gap`` noise units from its threshold (needs run_dmqr(...,
    margins=True)).  Within this prefix any backward-stable implementation
    must reproduce jpvt and the block sizes exactly."""
    bm = ref["block_margin"]
    nblk = int(np.count_nonzero(ref["ncols"])) if ref["ncols"][0] != 0 else 0
    b = 0
    while b < nblk and bm[b] >= gap:
        b += 1
    return b, int(np.sum(ref["ncols"][:b]))
