"""GPU QP3 (LAPACK dgeqp3 semantics), unpivoted QR (dgeqrf) and Q application
(dormqr 'L','N' / 'T') against LAPACK 3.12 through the oracle, plus the
fixed-column (jpvt != 0) pre-pass of dgeqrdm and dgeqp3.

QP3 pivots are compared over the separated prefix of steps: step i is
separated when the chosen pivot's partial norm exceeds every other
remaining partial norm by at least GAP_REL relatively and GAP_ABS noise
units (n eps ||A||_F) absolutely; partial norms are read off the final R
(||R(i:, j)|| for the pivoted column j).
"""
import numpy as np
import pytest

EPS = 2.0 ** -53
GAP_REL = 1e-6
GAP_ABS = 1e3


def qp3_separated_steps(A0, Rout):
    m, n = A0.shape
    k = min(m, n)
    R = np.triu(Rout[:k, :])
    noise = max(m, n) * EPS * np.linalg.norm(A0)
    # colnorm2[i, j] = ||R(i:, j)||^2 via reverse cumulative sums
    sq = R ** 2
    tail = np.cumsum(sq[::-1, :], axis=0)[::-1, :]
    steps = 0
    for i in range(k - 1):
        pn = np.sqrt(tail[i, i:])
        top = pn[0]
        rest = pn[1:].max() if pn.size > 1 else 0.0
        if top - rest < max(GAP_REL * top, GAP_ABS * noise):
            break
        steps += 1
    return steps


def gpu_qp3(A0, jpvt0=None):
    from qrdm_gb300 import QRDM

    A = np.array(A0, order="F", copy=True)
    m, n = A.shape
    jp = np.zeros(n, np.int32) if jpvt0 is None else np.array(jpvt0, np.int32)
    tau = np.zeros(min(m, n))
    info = QRDM.QP3(102, m, n, A, m, jp, tau)
    return A, jp, tau, info


def lapack_qp3(oracle, A0, jpvt0=None):
    A = np.array(A0, order="F", copy=True)
    m, n = A.shape
    jp = np.zeros(n, np.int32) if jpvt0 is None else np.array(jpvt0, np.int32)
    tau = np.zeros(min(m, n))
    info = oracle.dgeqp3(102, m, n, A, m, jp, tau)
    return A, jp, tau, info


def check_qr(A0, A, tau, jp, label):
    from qrdm_gb300.metrics import factor_metrics

    m, n = A0.shape
    met = factor_metrics(A0, A, tau, jp)
    bound = 10 * max(m, n) * EPS
    assert met["backward"] <= bound, (label, met)
    assert met["orth"] <= 10 * bound, (label, met)
    return met


@pytest.mark.gpu
def test_qp3_golden(gpu_lib, qp3_golden):
    for name, c in qp3_golden.items():
        A0 = np.asfortranarray(c["A_in"])
        A, jp, tau, info = gpu_qp3(A0)
        assert info == 0, name
        steps = qp3_separated_steps(A0, c["A_out"])
        assert np.array_equal(jp[:steps], c["jpvt"][:steps]), (name, steps)
        check_qr(A0, A, tau, jp, name)


@pytest.mark.gpu
@pytest.mark.parametrize("shape,seed", [((300, 200), 1), ((200, 300), 2), ((700, 500), 3),
                                        ((1000, 1000), 4)])
def test_qp3_vs_lapack(gpu_lib, oracle, shape, seed):
    from qrdm_gb300 import workloads as W

    m, n = shape
    A0 = W.gaussian(m, n, seed=seed) if seed % 2 else W.graded_svd(n, seed=seed)[:m, :] if m <= n \
        else W.gaussian(m, n, seed=seed)
    A0 = np.asfortranarray(A0)
    A, jp, tau, info = gpu_qp3(A0)
    Ar, jr, tr, ir = lapack_qp3(oracle, A0)
    assert info == ir == 0
    steps = qp3_separated_steps(A0, Ar)
    assert steps >= min(20, min(m, n) - 1)
    assert np.array_equal(jp[:steps], jr[:steps]), steps
    check_qr(A0, A, tau, jp, f"qp3 {shape}")


@pytest.mark.gpu
def test_qp3_fixed_columns(gpu_lib, oracle):
    from qrdm_gb300 import workloads as W

    A0 = W.gaussian(120, 90, seed=11)
    j0 = np.zeros(90, np.int32)
    j0[[3, 17, 40, 41]] = 1
    A, jp, tau, info = gpu_qp3(A0, j0)
    Ar, jr, tr, ir = lapack_qp3(oracle, A0, j0)
    assert info == ir == 0
    assert np.array_equal(jp[:4], jr[:4]) and sorted(jp[:4].tolist()) == [4, 18, 41, 42]
    steps = qp3_separated_steps(A0, Ar)
    assert np.array_equal(jp[:steps], jr[:steps])
    check_qr(A0, A, tau, jp, "qp3 fixed")


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(300, 200), (200, 300), (1000, 700), (64, 64), (5, 3)])
def test_dgeqrf_matches_lapack(gpu_lib, oracle, shape):
    from qrdm_gb300 import QRDM
    from qrdm_gb300 import workloads as W

    m, n = shape
    A0 = W.gaussian(m, n, seed=m + n)
    A = np.array(A0, order="F", copy=True)
    tau = np.zeros(min(m, n))
    assert QRDM.QRF(102, m, n, A, m, tau) == 0
    Ar = np.array(A0, order="F", copy=True)
    tr = np.zeros(min(m, n))
    assert oracle.dgeqrf(102, m, n, Ar, m, tr) == 0
    an = np.linalg.norm(A0)
    assert np.linalg.norm(np.triu(A) - np.triu(Ar)) <= 64 * max(m, n) * EPS * an
    assert np.max(np.abs(tau - tr)) <= 1e-10
    check_qr(A0, A, tau, np.arange(1, n + 1, dtype=np.int32), "qrf")


@pytest.mark.gpu
@pytest.mark.parametrize("k", [1, 37, 64, 130])
def test_dormqr_forms_q(gpu_lib, oracle, k):
    from qrdm_gb300 import QRDM
    from qrdm_gb300 import workloads as W

    m = 200
    A0 = W.gaussian(m, k, seed=k)
    A = np.array(A0, order="F", copy=True)
    tau = np.zeros(k)
    assert oracle.dgeqrf(102, m, k, A, m, tau) == 0
    Cg = np.asfortranarray(np.eye(m))
    assert QRDM.DORMQR(102, m, m, k, A, m, tau, Cg, m) == 0
    Cr = np.asfortranarray(np.eye(m))
    assert oracle.dormqr(102, m, m, k, A, m, tau, Cr, m) == 0
    assert np.linalg.norm(Cg - Cr) <= 100 * m * EPS
    assert np.linalg.norm(Cg.T @ Cg - np.eye(m)) <= 100 * m * EPS


@pytest.mark.gpu
def test_dgeqrdm_fixed_columns(gpu_lib, oracle):
    """jpvt != 0 columns go first, unpivoted (src/dgeqrdm_work.c:594-635);
    compared with the oracle's relative-index restatement."""
    import qrdm_gb300
    from oracle.oracle import run_dmqr, separated_prefix
    from qrdm_gb300 import workloads as W

    A0 = W.gaussian(150, 110, seed=12)
    j0 = np.zeros(110, np.int32)
    j0[[5, 60, 61]] = 1
    g = qrdm_gb300.dgeqrdm(A0, nb=16, jpvt=j0)
    r = run_dmqr(oracle, A0, nb=16, jpvt0=j0, margins=True)
    assert g["info"] == r["info"] == 0
    assert np.array_equal(g["jpvt"][:3], r["jpvt"][:3]) and sorted(g["jpvt"][:3]) == [6, 61, 62]
    nblk, cols = separated_prefix(r, 100.0)
    assert np.array_equal(g["jpvt"][3:3 + cols], r["jpvt"][3:3 + cols])
    from qrdm_gb300.metrics import factor_metrics

    met = factor_metrics(A0, g["A"], g["tau"], g["jpvt"])
    assert met["backward"] < 10 * 150 * EPS
