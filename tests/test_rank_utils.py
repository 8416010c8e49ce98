"""The auxil-style rank helpers (qrdm_gb300.rank) and the QR.py-style
DMrrqr adaptor (qrdm_gb300.qr_adaptor)."""
import numpy as np
import pytest

EPS = 2.0 ** -53


def test_rank_from_sv_convention():
    from qrdm_gb300.rank import rank_from_sv

    assert rank_from_sv([3.0, 2.0, 1.0]) == 3
    assert rank_from_sv([3.0, 2.0, 1e-12, 1e-13]) == 3  # 1-based position of the first small value
    assert rank_from_sv([1e-12, 2.0]) == 1
    assert rank_from_sv(np.array([1.0, -1e-10, 0.5]), tol=1e-9) == 2


def test_getR_layout():
    from qrdm_gb300.rank import getR

    rng = np.random.default_rng(0)
    m, n = 7, 5
    F = rng.standard_normal((m, n))
    At = np.ascontiguousarray(F.T)  # (n, m) convention
    assert np.array_equal(getR(102, m, n, At), np.triu(F))
    R3 = getR(102, m, n, At, k=3)
    assert np.array_equal(R3[:, :3], np.triu(F[:, :3]))
    assert np.array_equal(R3[:, 3:], F[:, 3:])
    with pytest.raises(ValueError):
        getR(101, m, n, At)


@pytest.mark.gpu
def test_checkQR_and_low_rank(gpu_lib):
    from qrdm_gb300 import QRDM
    from qrdm_gb300.rank import checkQR, low_rank, rank_from_sv
    from qrdm_gb300.workloads import rank_deficient_demo

    m = n = 96
    A0 = rank_deficient_demo(n, seed=3)
    Mt = np.ascontiguousarray(A0.T)  # (n, m) convention: column-major A0
    F = Mt.copy()
    jpvt = np.zeros(n, np.int32)
    tau = np.zeros(n)
    ncols = np.zeros(n, np.int32)
    assert QRDM.QRDM(102, m, n, F, m, jpvt, tau, ncols, np.array([0.9, 0.15]), 16) == 0
    Q, R, err, errQ = checkQR(102, m, n, F, Mt, tau, jpvt)
    an = np.linalg.norm(A0)
    assert err <= 10 * n * EPS * an and errQ <= 100 * n * EPS
    k = rank_from_sv(np.diag(R), tol=1e-9 * abs(R[0, 0])) - 1
    Ak = low_rank(102, m, n, F, Mt, tau, jpvt, k)
    p = jpvt - 1
    # rank-k truncation error equals ||R_22||
    assert abs(np.linalg.norm(A0[:, p] - Ak) - np.linalg.norm(R[k:, k:])) <= 1e3 * EPS * an


@pytest.mark.gpu
def test_dmrrqr_adaptor(gpu_lib):
    from qrdm_gb300.qr_adaptor import DMrrqr
    from qrdm_gb300.workloads import graded_svd

    A0 = graded_svd(120, seed=4)
    Q, R, piv, it = DMrrqr(A0, kDM=8, thres=0.5, thresnrm=0.3)
    assert sorted(piv.tolist()) == list(range(120))
    assert it >= 120 // 8
    an = np.linalg.norm(A0)
    assert np.linalg.norm(A0[:, piv] - Q @ R) <= 10 * 120 * EPS * an
    assert np.linalg.norm(np.eye(120) - Q.T @ Q) <= 100 * 120 * EPS
    assert np.allclose(R, np.triu(R))


def _auxil_checkQR(oracle, m, n, A, M, tau, jpvt, k=0):
    """auxil.checkQR (auxil.py:20-105) for matrix_layout 102, restated with
    the oracle's LAPACK DORMQR in place of QRDM.DORMQR: A, M in the (n, m)
    convention (C-ordered NumPy arrays whose buffers are column-major)."""
    mm, nn = (m, n) if m >= n else (m, m)
    min_mn = min(mm, nn)
    k = min_mn if (k == 0 or k > min_mn) else k
    Q = np.eye(m)
    assert oracle.dormqr(102, mm, nn, k, np.ascontiguousarray(A), m, np.asarray(tau, np.float64), Q, m) == 0
    if k == n:
        R = np.triu(A.T)
    else:
        R = np.zeros_like(A.T)
        R[:, :k] = np.triu(A[:k, :].T)
        R[:, k:] = A[k:, :].T
    Mt, Qt = M.T, Q.T
    errQ = np.linalg.norm(np.eye(m) - Qt.T @ Qt)
    err = np.linalg.norm(Mt[:, jpvt - 1] - Qt @ R)
    return Qt, R, err, errQ


def _auxil_low_rank(oracle, m, n, M, tau, k):
    """auxil.low_rank (auxil.py:156-200), layout 102, with the oracle's
    DORMQR."""
    min_mn = min(m, n)
    k = min_mn if (k == 0 or k > min_mn) else k
    if k == n:
        R = np.tril(M)
    else:
        R = np.zeros_like(M)
        R[:k, :] = np.tril(M[:k, :])
        R[k:, :k] = M[k:, :k]
    Alow = np.ascontiguousarray(R.copy())
    assert oracle.dormqr(102, m, n, k, np.ascontiguousarray(M), m, np.asarray(tau, np.float64), Alow, m) == 0
    return Alow.T


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(160, 160), (300, 120)])
def test_device_helpers_match_auxil_formulas(gpu_lib, oracle, shape):
    """checkQR_dev / low_rank_dev / apply_jpvt_dev against the reference's
    auxil formulas evaluated with the oracle's LAPACK DORMQR on the same
    factorisation: Q and the rank-k approximation agree to rounding, A P is
    exact, err agrees (and errQ where auxil forms all of Q, m == n)."""
    import torch

    import qrdm_gb300
    from qrdm_gb300.rank import apply_jpvt_dev, checkQR_dev, low_rank_dev
    from qrdm_gb300.workloads import graded_svd, low_rank_noise

    m, n = shape
    A0 = graded_svd(n, seed=6) if m == n else low_rank_noise(m, n, r=40, noise=1e-9, seed=7)
    res = qrdm_gb300.dgeqrdm(A0, nb=32)
    assert res["info"] == 0
    F = np.ascontiguousarray(res["A"].T)  # (n, m) convention
    Mt = np.ascontiguousarray(A0.T)
    tau, jpvt = res["tau"], res["jpvt"]
    an = np.linalg.norm(A0)
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    Fd, Md, taud, jpd = dev(F), dev(Mt), dev(tau), dev(jpvt.astype(np.int32))
    # A P: an exact gather
    AP = apply_jpvt_dev(m, n, Md, jpd).cpu().numpy().T
    assert np.array_equal(AP, A0[:, jpvt - 1])
    Qd, Rd, err, errQ = checkQR_dev(102, m, n, Fd, Md, taud, jpd)
    Qr, Rr, err_r, errQ_r = _auxil_checkQR(oracle, m, n, F, Mt, tau, jpvt)
    Q = Qd.cpu().numpy().T
    assert np.array_equal(Rd.cpu().numpy().T, Rr)
    nq = min(m, n)  # the columns auxil.checkQR forms
    assert np.linalg.norm(Q[:, :nq] - Qr[:, :nq]) <= 100 * m * EPS
    assert abs(err - err_r) <= 10 * max(m, n) * EPS * an and err <= 10 * max(m, n) * EPS * an
    if m == n:
        assert errQ <= 100 * m * EPS and errQ_r <= 100 * m * EPS
        assert abs(errQ - errQ_r) <= 100 * m * EPS
    else:  # all m columns of Q are orthonormal here (auxil leaves m - n of them unit vectors)
        assert errQ <= 100 * m * EPS
    k = max(1, int(np.count_nonzero(np.abs(np.diag(res["A"])) > 1e-6 * abs(res["A"][0, 0]))))
    Ak = low_rank_dev(102, m, n, Fd, Md, taud, jpd, k).cpu().numpy()
    Ak_r = _auxil_low_rank(oracle, m, n, F, tau, k)
    assert np.linalg.norm(Ak - Ak_r) <= 100 * max(m, n) * EPS * an


@pytest.mark.gpu
def test_norm_diff_and_gather_arguments(gpu_lib):
    import ctypes as C

    import torch

    L = gpu_lib
    x = torch.randn(37, 53, dtype=torch.float64, device="cuda")
    y = torch.randn(37, 53, dtype=torch.float64, device="cuda")
    out = C.c_double(0.0)
    assert L.qrdm_norm_diff_dev(53, 37, C.c_void_p(x.data_ptr()), 53, C.c_void_p(y.data_ptr()), 53,
                                C.byref(out)) == 0
    ref = float(torch.linalg.norm(x - y))
    assert abs(out.value - ref) <= 1e-13 * ref
    assert L.qrdm_norm_diff_dev(53, 37, C.c_void_p(x.data_ptr()), 53, None, 53, C.byref(out)) == 0
    assert abs(out.value - float(torch.linalg.norm(x))) <= 1e-13 * float(torch.linalg.norm(x))
    bad = torch.tensor([1, 2, 99], dtype=torch.int32, device="cuda")
    o = torch.empty(3, 4, dtype=torch.float64, device="cuda")
    a = torch.zeros(3, 4, dtype=torch.float64, device="cuda")
    assert L.qrdm_apply_jpvt_dev(4, 3, C.c_void_p(a.data_ptr()), 4, C.c_void_p(bad.data_ptr()),
                                 C.c_void_p(o.data_ptr()), 4) == -5
