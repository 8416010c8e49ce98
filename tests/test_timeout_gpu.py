"""The bounded-wait path: every device-wide wait of the library gives up
after a bounded number of polls, reports QRDM_ERR_TIMEOUT (1002) and leaves
the process usable.  The reference has no device waits; this extends its
info convention (0 / -1 / LAPACKE codes, src/dgeqrdm_work.c:559-589,
:743-771) with a positive code.

The wait is made to run out without any fault: qrdm_options.wait_limit = 1
lets each panel CTA poll its grid barrier once before giving up, so a
factorisation whose panel spans many CTAs stops at its first DM block.  The
kernels return normally (the panel CTAs break out of their loops, the rest
of the block sees fjb_cmp = 0 and does nothing), and the next call with the
default limit must succeed with bit-identical results."""
import ctypes as C

import numpy as np
import pytest


def _factor(L, at, n, m, wait_limit=0, precision=0):
    import torch

    from qrdm_gb300 import Stats, default_options

    a = at.clone()
    jp = torch.zeros(n, dtype=torch.int32, device="cuda")
    tau = torch.zeros(min(m, n), dtype=torch.float64, device="cuda")
    nc = np.zeros(n, np.int32)
    thres = np.array([0.9, 0.15, 0.0])
    opt = default_options(precision=precision, wait_limit=wait_limit)
    st = Stats()
    torch.cuda.synchronize()
    info = L.dgeqrdm_dev(102, m, n, C.c_void_p(a.data_ptr()), m, C.c_void_p(jp.data_ptr()),
                         C.c_void_p(tau.data_ptr()), nc.ctypes.data_as(C.POINTER(C.c_int)),
                         thres.ctypes.data_as(C.POINTER(C.c_double)), 64, C.byref(opt), C.byref(st))
    torch.cuda.synchronize()
    return info, a, jp, tau, nc


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_panel_wait_gives_up_and_the_next_call_is_exact(gpu_lib, precision):
    import torch

    from qrdm_gb300 import workloads as W

    L = gpu_lib
    L.qrdm_set_stream(None)
    m, n = 4096, 320  # panels of 4096 rows: 64 CTAs meet at every grid barrier
    at = torch.from_numpy(np.ascontiguousarray(W.gaussian(m, n, seed=23).T)).cuda()
    info0, a0, jp0, tau0, nc0 = _factor(L, at, n, m, precision=precision)
    assert info0 == 0
    info1, *_ = _factor(L, at, n, m, wait_limit=1, precision=precision)
    assert info1 == 1002  # QRDM_ERR_TIMEOUT
    info2, a2, jp2, tau2, nc2 = _factor(L, at, n, m, precision=precision)
    assert info2 == 0
    assert torch.equal(a2, a0) and torch.equal(jp2, jp0) and torch.equal(tau2, tau0)
    assert np.array_equal(nc2, nc0)


@pytest.mark.gpu
def test_negative_wait_limit_is_an_invalid_argument(gpu_lib):
    import torch

    L = gpu_lib
    at = torch.zeros(8, 16, dtype=torch.float64, device="cuda")
    info, *_ = _factor(L, at, 8, 16, wait_limit=-5)
    assert info == -1
