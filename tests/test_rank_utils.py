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
