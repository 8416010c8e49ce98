"""Mixed-precision DM-QR: the trailing update on FP16 tensor cores through an
Ozaki split (FP64 emulation).  Same parity bar as the FP64 path: identical
jpvt / DM blocks over the gap-separated prefix of the oracle's run, backward
error <= 10 max(m,n) eps, orthogonality <= 100 max(m,n) eps."""
import numpy as np
import pytest

EPS = 2.0 ** -53
GAP = 100.0


def run(A0, precision, nb=64, **kw):
    import qrdm_gb300

    return qrdm_gb300.dgeqrdm(A0, nb=nb, precision=precision, **kw)


def check(oracle, A0, r, nb=64, label=""):
    from oracle.oracle import run_dmqr, separated_prefix
    from qrdm_gb300.metrics import factor_metrics

    m, n = A0.shape
    ref = run_dmqr(oracle, A0, nb=nb, margins=True)
    nblk, cols = separated_prefix(ref, GAP)
    assert r["info"] == 0, (label, r["info"])
    assert np.array_equal(r["ncols"][:nblk], ref["ncols"][:nblk]), (label, nblk)
    assert np.array_equal(r["jpvt"][:cols], ref["jpvt"][:cols]), (label, cols)
    met = factor_metrics(A0, r["A"], r["tau"], r["jpvt"])
    assert met["backward"] <= 10 * max(m, n) * EPS, (label, met["backward"])
    assert met["orth"] <= 100 * max(m, n) * EPS, (label, met["orth"])
    return met, nblk, cols


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["gauss500x400", "graded1000", "lowrank1500x900", "wide300x700",
                                  "tall2100x260"])
def test_mixed_dmqr_parity(gpu_lib, oracle, case):
    from qrdm_gb300 import workloads as W

    A0 = {"gauss500x400": lambda: W.gaussian(500, 400, seed=41),
          "graded1000": lambda: W.graded_svd(1000, seed=0),
          "lowrank1500x900": lambda: W.low_rank_noise(1500, 900, 200, 1e-10, seed=42),
          "wide300x700": lambda: W.gaussian(300, 700, seed=43),
          "tall2100x260": lambda: W.gaussian(2100, 260, seed=44)}[case]()
    r = run(A0, "mixed")
    met, nblk, cols = check(oracle, A0, r, label=case)
    f = run(A0, "fp64")
    # the two GPU precisions agree on the separated prefix as well
    assert np.array_equal(r["jpvt"][:cols], f["jpvt"][:cols])


@pytest.mark.gpu
@pytest.mark.parametrize("slices", [5, 6, 7])
def test_mixed_slices(gpu_lib, oracle, slices):
    from qrdm_gb300 import workloads as W
    from qrdm_gb300._lib import Stats, default_options, lib
    import ctypes as C

    A0 = W.gaussian(400, 300, seed=50 + slices)
    A = np.array(A0, order="F", copy=True)
    m, n = A.shape
    jp = np.zeros(n, np.int32)
    tau = np.zeros(n)
    nc = np.zeros(n, np.int32)
    th = np.array([0.9, 0.15, 0.0])
    opt = default_options(precision=1, slices=slices)
    pd, pi = C.POINTER(C.c_double), C.POINTER(C.c_int)
    info = lib().dgeqrdm_ex(102, m, n, A.ctypes.data_as(pd), m, jp.ctypes.data_as(pi),
                            tau.ctypes.data_as(pd), nc.ctypes.data_as(pi), th.ctypes.data_as(pd),
                            64, C.byref(opt), None)
    assert info == 0
    from qrdm_gb300.metrics import factor_metrics

    met = factor_metrics(A0, A, tau, jp)
    # error of the split ~ 2^-(8 s - 8) relative; 7 slices are FP64-grade
    bound = {5: 1e-9, 6: 1e-11, 7: 10 * 400 * EPS}[slices]
    assert met["backward"] <= bound, (slices, met["backward"])


@pytest.mark.gpu
def test_mixed_gram_recheck_near_delta(gpu_lib, oracle):
    """Pairs of columns with cosines 0.9 +- 0.002 straddle delta = 0.9 closer
    than the BF16 cosine error (~2^-8): the FP64 recheck must reproduce the
    reference's accept/reject decisions."""
    import qrdm_gb300

    rng = np.random.default_rng(77)
    m, n = 600, 160
    A0 = rng.standard_normal((m, n))
    A0 /= np.linalg.norm(A0, axis=0)
    for t in range(0, n, 2):
        a = A0[:, t]
        z = rng.standard_normal(m)
        z -= a * (a @ z)
        z /= np.linalg.norm(z)
        c = 0.9 + (0.002 if (t // 2) % 2 == 0 else -0.002)
        A0[:, t + 1] = c * a + np.sqrt(1 - c * c) * z
    A0 *= 1.0 + 0.05 * rng.standard_normal(n)  # distinct norms
    A0 = np.asfortranarray(A0)
    r = run(A0, "mixed")
    met, nblk, cols = check(oracle, A0, r, label="recheck")
    assert nblk >= 1 and cols >= 20
    assert r["stats"]["rechecks"] > 0
