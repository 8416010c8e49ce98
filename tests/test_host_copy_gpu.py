"""dgeqrdm_ex's host copies: a page-locked host matrix receives its finished
columns while later DM blocks still run (a second stream, behind each
block's kernels); a pageable one is copied once at the end.  Both must give
the same bits, with lda = m and with a padded lda, and with a stop that
leaves unfactored columns."""
import ctypes as C

import numpy as np
import pytest


def _ex(A_store, m, n, lda, stop=0, precision=0):
    from qrdm_gb300 import Stats, default_options, lib

    jp = np.zeros(n, np.int32)
    tau = np.zeros(min(m, n))
    nc = np.zeros(n, np.int32)
    nc[0] = stop
    thres = np.array([0.9, 0.15, 1e-6])
    opt = default_options(precision=precision)
    st = Stats()
    pd, pi = C.POINTER(C.c_double), C.POINTER(C.c_int)
    info = lib().dgeqrdm_ex(102, m, n, A_store.ctypes.data_as(pd), lda, jp.ctypes.data_as(pi),
                            tau.ctypes.data_as(pd), nc.ctypes.data_as(pi), thres.ctypes.data_as(pd), 64,
                            C.byref(opt), C.byref(st))
    return info, jp, tau, nc


@pytest.mark.gpu
@pytest.mark.parametrize("pad,stop,precision", [(0, 0, 0), (5, 0, 1), (0, 3, 1)])
def test_pinned_and_pageable_host_buffers_agree(gpu_lib, pad, stop, precision):
    import torch

    from qrdm_gb300 import workloads as W

    m, n = 2500, 1800
    A0 = W.low_rank_noise(m, n, r=600, noise=1e-9, seed=31) if stop else W.gaussian(m, n, seed=31)
    lda = m + pad
    pageable = np.zeros((n, lda))
    pageable[:, :m] = A0.T
    pinned_t = torch.empty((n, lda), dtype=torch.float64, pin_memory=True)
    pinned = pinned_t.numpy()
    pinned[...] = pageable
    r1 = _ex(pageable, m, n, lda, stop, precision)
    r2 = _ex(pinned, m, n, lda, stop, precision)
    assert r1[0] == 0 and r2[0] == 0
    for x, y in zip(r1[1:], r2[1:]):
        assert np.array_equal(x, y)
    assert np.array_equal(pageable, pinned)  # every column, padding untouched
    if stop:
        assert int(np.sum(r1[3])) < min(m, n)  # the stop left columns unfactored
