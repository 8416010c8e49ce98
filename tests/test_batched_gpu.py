"""Batched DM-QR (dgeqrdm_batched_dev): many uneven problems in one
persistent kernel, each held to the single-problem parity bar against the
oracle (jpvt and block sizes over the gap-separated prefix, leading R block,
backward error <= 10 max(m,n) eps; see test_dmqr_gpu.py)."""
import numpy as np
import pytest

from test_dmqr_gpu import check_against, separated

P = (0.9, 0.15, 32, 0, None)  # delta, tau_, nb, stop, eta


def _mixed_batch():
    from qrdm_gb300.workloads import batched_matrix, batched_shapes, gaussian, rank_deficient_demo

    ms, ns = batched_shapes(count=20, seed=11, nmin=8, nmax=200, mcap=600)
    mats = [batched_matrix(i, int(m), int(n), seed=11) for i, (m, n) in enumerate(zip(ms, ns))]
    rng = np.random.default_rng(3)
    mats += [
        rng.standard_normal((1, 1)),
        rng.standard_normal((5, 1)),
        rng.standard_normal((1, 7)),
        rng.standard_normal((3, 9)),       # wide
        rng.standard_normal((40, 96)),     # wide, more columns than rows
        gaussian(70, 70, seed=5),
        rank_deficient_demo(64, seed=2),
        np.zeros((12, 6)),                 # all-zero columns
    ]
    return mats


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_uneven_vs_oracle(gpu_lib, oracle, precision):
    import qrdm_gb300

    mats = _mixed_batch()
    out = qrdm_gb300.dgeqrdm_batched(mats, nb=32, delta=0.9, tau_=0.15, precision=precision)
    assert len(out) == len(mats)
    for i, A0 in enumerate(mats):
        prefix, ref = separated(oracle, A0, P)
        check_against(A0, out[i], ref, prefix, f"batched[{i}] {A0.shape} {precision}")


@pytest.mark.gpu
@pytest.mark.parametrize("nb,precision", [(8, "fp64"), (64, "fp64"), (8, "mixed"), (16, "mixed")])
def test_batched_block_sizes(gpu_lib, oracle, nb, precision):
    import qrdm_gb300
    from qrdm_gb300.workloads import batched_matrix

    shapes = [(300, 200), (128, 128), (513, 257), (65, 65), (90, 33), (1100, 700)]
    mats = [batched_matrix(i, m, n, seed=21) for i, (m, n) in enumerate(shapes)]
    out = qrdm_gb300.dgeqrdm_batched(mats, nb=nb, delta=0.5, tau_=0.3, precision=precision)
    p = (0.5, 0.3, nb, 0, None)
    for i, A0 in enumerate(mats):
        prefix, ref = separated(oracle, A0, p)
        check_against(A0, out[i], ref, prefix, f"nb={nb} [{i}]")


@pytest.mark.gpu
@pytest.mark.parametrize("stop,eta,precision", [(1, None, "fp64"), (2, None, "fp64"), (3, 1e-6, "fp64"),
                                                (1, None, "mixed")])
def test_batched_stop_modes(gpu_lib, oracle, stop, eta, precision):
    import qrdm_gb300
    from qrdm_gb300.workloads import rank_deficient_demo

    mats = [rank_deficient_demo(96, seed=s) for s in range(4)]
    out = qrdm_gb300.dgeqrdm_batched(mats, nb=16, delta=0.9, tau_=0.15, stop=stop, eta=eta,
                                     precision=precision)
    p = (0.9, 0.15, 16, stop, eta)
    for i, A0 in enumerate(mats):
        prefix, ref = separated(oracle, A0, p)
        check_against(A0, out[i], ref, prefix, f"stop={stop} [{i}]")
        # a stopped factorisation covers fewer than n columns
        if prefix[0] == int(np.count_nonzero(ref["ncols"])):
            assert out[i]["nblocks"] == int(np.count_nonzero(ref["ncols"]))


@pytest.mark.gpu
def test_batched_graph_replay(gpu_lib, oracle):
    """A repeated call with the same description replays the captured launch
    on new data and still gives the right answers."""
    from qrdm_gb300 import BatchedDMQR
    from qrdm_gb300.workloads import batched_matrix

    shapes = [(200, 150), (64, 64), (400, 100), (33, 17)]
    b = BatchedDMQR(shapes)
    for seed, prec in ((31, "fp64"), (32, "fp64"), (33, "mixed"), (34, "mixed")):
        mats = [batched_matrix(i, m, n, seed=seed) for i, (m, n) in enumerate(shapes)]
        b.load(mats)
        assert b.run(nb=32, precision=prec) == 0
        out = b.results()
        for i, A0 in enumerate(mats):
            prefix, ref = separated(oracle, A0, P)
            check_against(A0, out[i], ref, prefix, f"replay seed={seed} {prec} [{i}]")


@pytest.mark.gpu
def test_batched_nan_problem(gpu_lib, oracle):
    import qrdm_gb300

    rng = np.random.default_rng(9)
    mats = [rng.standard_normal((50, 40)) for _ in range(3)]
    mats[1][7, 3] = np.nan
    out = qrdm_gb300.dgeqrdm_batched(mats, nb=32)
    assert [o["info"] for o in out] == [0, -13, 0]
    for i in (0, 2):
        prefix, ref = separated(oracle, mats[i], P)
        check_against(mats[i], out[i], ref, prefix, f"nan-batch [{i}]")


@pytest.mark.gpu
def test_batched_argument_errors(gpu_lib):
    import ctypes as C

    from qrdm_gb300 import BatchedDMQR

    b = BatchedDMQR([(8, 8)])
    assert b.run(nb=65) == 1003          # nb beyond the batched kernel
    assert b.run(nb=64, precision="mixed") == 1003  # mixed: nb <= 32
    assert b.run(nb=0) == -1
    assert b.run(nb=8, delta=1.5) == -1
    assert b.run(nb=8, stop=4) == -1
    big = BatchedDMQR([(4, 1025)])
    assert big.run(nb=8) == 1003         # n beyond the batched kernel
    thres = (C.c_double * 3)(0.9, 0.15, 0.0)
    assert gpu_lib.dgeqrdm_batched_dev(0, None, None, None, None, None, None, None, thres, 0, 8, 0) == -1
    m = (C.c_int * 1)(0)
    n = (C.c_int * 1)(4)
    assert gpu_lib.dgeqrdm_batched_dev(1, m, n, None, None, None, None, None, thres, 0, 8, 0) == -1
    assert gpu_lib.dgeqrdm_batched_dev(1, m, n, None, None, None, None, None, thres, 0, 8, 2) == -1


@pytest.mark.gpu
def test_batched_autotune(gpu_lib):
    """The autotuner times its candidates on the batch's shapes and returns
    one of them; the chosen configuration factors the batch correctly."""
    import qrdm_gb300
    from qrdm_gb300.autotune import DEFAULT_CANDIDATES, tune_batched
    from qrdm_gb300.metrics import factor_metrics
    from qrdm_gb300.workloads import batched_matrix, batched_shapes

    ms, ns = batched_shapes(count=40, seed=13, nmin=16, nmax=160, mcap=400)
    shapes = [(int(m), int(n)) for m, n in zip(ms, ns)]
    t = tune_batched(shapes, sample=None, reps=1)
    assert (t["nb"], t["precision"]) in DEFAULT_CANDIDATES
    assert all(v < float("inf") for v in t["ms"].values()), t
    assert tune_batched(shapes, sample=None, reps=1) is t  # cached per signature
    mats = [batched_matrix(i, m, n, seed=13) for i, (m, n) in enumerate(shapes)]
    out = qrdm_gb300.dgeqrdm_batched(mats, nb=t["nb"], precision=t["precision"])
    for A0, r in zip(mats, out):
        met = factor_metrics(A0, r["A"], r["tau"], r["jpvt"])
        assert met["backward"] <= 10 * max(A0.shape) * 2.0 ** -53
