"""dgeqrdm_dev_noalloc: DM-QR for callers that cannot allocate device memory
(plug-ins whose host application owns every device allocation, real-time
loops that cannot take cudaMalloc's implicit synchronisation, processes at
their memory limit).  All of its scratch lives in a fixed device array
inside the library, so it must agree with the allocating entry point
dgeqrdm_dev -- on consecutive calls too, since each call inherits the
array's previous contents -- on the caller's own stream and with fixed
columns (which run the unpivoted pre-factorisation out of the same array).
Collected last on purpose (tests/test_zz_*)."""
import ctypes as C

import numpy as np
import pytest

EPS = 2.0 ** -53
RTOL_R = 64.0  # the R tolerance of the DM-QR parity tests


def _run(entry, A0, nb, stream=None, jpvt0=None):
    import torch

    m, n = A0.shape
    a = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()  # column-major m x n
    jp0 = np.zeros(n, np.int32) if jpvt0 is None else np.asarray(jpvt0, np.int32)
    jp = torch.from_numpy(jp0.copy()).cuda()
    tau = torch.zeros(min(m, n), dtype=torch.float64, device="cuda")
    ncols = np.zeros(n, np.int32)
    thres = np.array([0.9, 0.15, 0.0])
    torch.cuda.synchronize()  # inputs complete before a call on another stream
    pi, pd = C.POINTER(C.c_int), C.POINTER(C.c_double)
    args = [102, m, n, C.c_void_p(a.data_ptr()), m, C.c_void_p(jp.data_ptr()),
            C.c_void_p(tau.data_ptr()), ncols.ctypes.data_as(pi), thres.ctypes.data_as(pd), nb]
    if entry.__name__ == "dgeqrdm_dev_noalloc":
        args.append(C.c_void_p(stream))
    else:
        args += [None, None]
    info = entry(*args)
    torch.cuda.synchronize()
    return {"info": info, "A": a.cpu().numpy().T, "jpvt": jp.cpu().numpy(),
            "tau": tau.cpu().numpy(), "ncols": ncols}


def _same(got, ref, A0):
    assert ref["info"] == 0 and got["info"] == 0, (ref["info"], got["info"])
    assert np.array_equal(got["jpvt"], ref["jpvt"])
    assert np.array_equal(got["ncols"], ref["ncols"])
    an = np.linalg.norm(A0)
    n = A0.shape[1]
    assert np.linalg.norm(np.triu(got["A"]) - np.triu(ref["A"])) <= RTOL_R * n * EPS * an
    assert np.max(np.abs(got["tau"] - ref["tau"])) <= RTOL_R * n * EPS


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_on_two_calls(gpu_lib):
    from qrdm_gb300 import workloads as W

    L = gpu_lib
    cases = [(W.graded_svd(600, seed=5), 64), (W.gaussian(1024, 700, seed=6), 32)]
    for A0, nb in cases:  # two calls in a row, different shapes and contents
        ref = _run(L.dgeqrdm_dev, A0, nb)
        got = _run(L.dgeqrdm_dev_noalloc, A0, nb)
        _same(got, ref, A0)


@pytest.mark.gpu
def test_noalloc_on_caller_stream_with_fixed_columns(gpu_lib):
    """The caller's own stream, and jpvt marking fixed leading columns
    (moved to the front, factored without pivoting, Q^T applied to the
    rest, all with the static scratch)."""
    import torch

    from qrdm_gb300 import workloads as W

    L = gpu_lib
    A0 = W.gaussian(800, 500, seed=11)
    jp0 = np.zeros(500, np.int32)
    jp0[[3, 10, 77, 499]] = 1
    side = torch.cuda.Stream()
    for _ in range(2):  # twice: the second call starts from the first's leftovers
        ref = _run(L.dgeqrdm_dev, A0, 64, jpvt0=jp0)
        got = _run(L.dgeqrdm_dev_noalloc, A0, 64, stream=side.cuda_stream, jpvt0=jp0)
        _same(got, ref, A0)
        assert sorted(got["jpvt"][:4]) == [4, 11, 78, 500]


@pytest.mark.gpu
def test_noalloc_rejects_sizes_beyond_its_scratch(gpu_lib):
    import torch

    L = gpu_lib
    m, n = 2048, 64
    a = torch.zeros(n, m, dtype=torch.float64, device="cuda")
    jp = torch.zeros(n, dtype=torch.int32, device="cuda")
    tau = torch.zeros(n, dtype=torch.float64, device="cuda")
    ncols = np.zeros(n, np.int32)
    thres = np.array([0.9, 0.15, 0.0])
    pi, pd = C.POINTER(C.c_int), C.POINTER(C.c_double)
    rc = L.dgeqrdm_dev_noalloc(102, m, n, C.c_void_p(a.data_ptr()), m, C.c_void_p(jp.data_ptr()),
                               C.c_void_p(tau.data_ptr()), ncols.ctypes.data_as(pi),
                               thres.ctypes.data_as(pd), 64, None)
    assert rc == 1003  # QRDM_ERR_UNSUPPORTED
    rc = L.dgeqrdm_dev_noalloc(102, 0, n, C.c_void_p(a.data_ptr()), 1, C.c_void_p(jp.data_ptr()),
                               C.c_void_p(tau.data_ptr()), ncols.ctypes.data_as(pi),
                               thres.ctypes.data_as(pd), 64, None)
    assert rc == -1  # invalid shape, rejected before any workspace is touched
