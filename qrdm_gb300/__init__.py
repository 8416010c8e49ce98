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
    import torch

    n, m = a.shape
    lib().qrdm_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
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


class BatchedDMQR:
    """Device-resident batch of uneven DM-QR problems for
    ``dgeqrdm_batched_dev``: matrices packed column-major in one float64
    CUDA buffer (problem i at ``a_off[i]`` with lda = m_i), jpvt / ncols at
    ``v_off[i]``, tau at ``t_off[i]``.  ``load`` copies host matrices in,
    ``run`` factors all of them with one persistent kernel launch (replayed
    from a CUDA graph when the description repeats), ``result(i)`` reads one
    problem back."""

    def __init__(self, shapes, device="cuda"):
        import torch
        self.shapes = [(int(m), int(n)) for m, n in shapes]
        self.count = len(self.shapes)
        self.m = np.array([s[0] for s in self.shapes], np.int32)
        self.n = np.array([s[1] for s in self.shapes], np.int32)
        mn = self.m.astype(np.int64) * self.n
        self.a_off = np.concatenate([[0], np.cumsum(mn)]).astype(np.int64)
        self.v_off = np.concatenate([[0], np.cumsum(self.n)]).astype(np.int64)
        self.t_off = np.concatenate([[0], np.cumsum(np.minimum(self.m, self.n))]).astype(np.int64)
        self.a = torch.zeros(int(self.a_off[-1]), dtype=torch.float64, device=device)
        self.jpvt = torch.zeros(int(self.v_off[-1]), dtype=torch.int32, device=device)
        self.ncols = torch.zeros(int(self.v_off[-1]), dtype=torch.int32, device=device)
        self.tau = torch.zeros(max(1, int(self.t_off[-1])), dtype=torch.float64, device=device)
        self.info = torch.zeros(max(1, self.count), dtype=torch.int32, device=device)

    def pack(self, mats) -> np.ndarray:
        """Host array holding the matrices in the device layout."""
        buf = np.empty(int(self.a_off[-1]), np.float64)
        for i, A in enumerate(mats):
            m, n = self.shapes[i]
            buf[self.a_off[i]:self.a_off[i + 1]] = np.asarray(A, np.float64).reshape(m, n).ravel(order="F")
        return buf

    def load(self, mats):
        import torch
        self.a.copy_(torch.from_numpy(self.pack(mats)))

    def run(self, nb: int = 32, delta: float = 0.9, tau_: float = 0.15, stop: int = 0,
            eta: float | None = None, precision: str = "fp64") -> int:
        import torch

        thres = np.array([delta, tau_, 0.0 if eta is None else eta], np.float64)
        lib().qrdm_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
        return int(lib().dgeqrdm_batched_dev(
            self.count, self.m.ctypes.data_as(C.POINTER(C.c_int)),
            self.n.ctypes.data_as(C.POINTER(C.c_int)), C.c_void_p(self.a.data_ptr()),
            C.c_void_p(self.jpvt.data_ptr()), C.c_void_p(self.tau.data_ptr()),
            C.c_void_p(self.ncols.data_ptr()), C.c_void_p(self.info.data_ptr()),
            thres.ctypes.data_as(C.POINTER(C.c_double)), int(stop), int(nb), PREC[precision]))

    def results(self) -> list:
        a = self.a.cpu().numpy()
        jp = self.jpvt.cpu().numpy()
        nc = self.ncols.cpu().numpy()
        tau = self.tau.cpu().numpy()
        info = self.info.cpu().numpy()
        out = []
        for i, (m, n) in enumerate(self.shapes):
            blocks = nc[self.v_off[i]:self.v_off[i + 1]]
            out.append({
                "A": a[self.a_off[i]:self.a_off[i + 1]].reshape(n, m).T.copy(),
                "jpvt": jp[self.v_off[i]:self.v_off[i + 1]].copy(),
                "ncols": blocks.copy(),
                "nblocks": int(np.count_nonzero(blocks)),
                "tau": tau[self.t_off[i]:self.t_off[i + 1]].copy(),
                "info": int(info[i]),
            })
        return out


def dgeqrdm_batched(mats, nb: int = 32, delta: float = 0.9, tau_: float = 0.15, stop: int = 0,
                    eta: float | None = None, precision: str = "fp64") -> list:
    """Factor a list of host matrices (uneven shapes, n <= 1024) with one
    batched DM-QR launch; returns one result dict per matrix."""
    mats = [np.asarray(A, np.float64) for A in mats]
    b = BatchedDMQR([A.shape for A in mats])
    b.load(mats)
    r = b.run(nb=nb, delta=delta, tau_=tau_, stop=stop, eta=eta, precision=precision)
    if r != 0:
        raise RuntimeError(f"dgeqrdm_batched_dev failed: {r}")
    return b.results()


__all__ = ["dgeqrdm", "dgeqrdm_device", "dgeqrdm_batched", "BatchedDMQR", "Options", "Stats", "default_options", "lib", "PREC"]
