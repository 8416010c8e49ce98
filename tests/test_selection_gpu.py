"""Selection-stress DM-QR (column-subset selection, stopped after k columns):
wide matrices whose base columns are repeated up to 8 times with a 1e-8
relative perturbation, plus filler columns of graded size.

Copies of one base column have norms within ~1e-8 of each other, so which
copy comes first is a near-tie that any rounding difference may flip; the
copies are interchangeable for the selection.  Parity with the oracle on the
same input is therefore checked on column identities (the base index of a
copy, the column index of a filler column): the DM block sizes, and each
block's set of identities, over the blocks that reach k.  Also: the
backward error of the stopped factorisation, and the size-independent
property that no two of the first k selected columns are copies of the same
base column (a copy's residual after its base is taken is ~1e-8 of its
norm)."""
import numpy as np
import pytest

EPS = 2.0 ** -53


def _case(m, n, nbase, seed):
    from qrdm_gb300.workloads import selection_stress

    return selection_stress(m=m, n=n, nbase=nbase, seed=seed, return_base=True)


def _ident(jpvt, bid):
    b = bid[jpvt - 1]
    return np.where(b >= 0, b, -1 - (jpvt - 1).astype(np.int64))


def _blocks(ncols, kstop):
    nb = 0
    tot = 0
    while nb < len(ncols) and ncols[nb] > 0 and tot < kstop:
        tot += int(ncols[nb])
        nb += 1
    return nb, tot


def _check_selection(A0, bid, gpu, kstop, label):
    from qrdm_gb300.metrics import factor_metrics

    assert gpu["info"] == 0, label
    nb, k = _blocks(gpu["ncols"], kstop)
    assert k >= kstop, (label, k)
    sel = bid[gpu["jpvt"][:kstop] - 1]
    sel = sel[sel >= 0]
    assert len(np.unique(sel)) == len(sel), (label, "a base column was selected twice")
    m, n = A0.shape
    met = factor_metrics(A0, gpu["A"], gpu["tau"], gpu["jpvt"], k=k)
    assert met["backward"] <= 10 * max(m, n) * EPS, (label, met["backward"])
    return nb, k


@pytest.mark.gpu
@pytest.mark.parametrize("m,n,nbase,kstop,seed", [(384, 1536, 192, 192, 5), (256, 2048, 128, 128, 6)])
def test_selection_stress_vs_oracle(gpu_lib, oracle, m, n, nbase, kstop, seed):
    import qrdm_gb300
    from oracle.oracle import run_dmqr

    A0, bid = _case(m, n, nbase, seed)
    ref = run_dmqr(oracle, A0, delta=0.9, tau_=0.15, nb=64, kstop=kstop, margins=True)
    # the decisions other than the copies' order are far from their thresholds
    for key in ("candidate", "cosine", "panel_exit"):
        assert ref["margins"][key] >= 100.0, (key, ref["margins"][key])
    nbr, kr = _blocks(ref["ncols"], kstop)
    for prec in ("mixed", "fp64"):
        gpu = qrdm_gb300.dgeqrdm(A0, nb=64, delta=0.9, tau_=0.15, precision=prec, kstop=kstop)
        nb, k = _check_selection(A0, bid, gpu, kstop, f"{m}x{n} {prec}")
        assert (nb, k) == (nbr, kr), (prec, nb, k, nbr, kr)
        assert np.array_equal(gpu["ncols"][:nb], ref["ncols"][:nb]), prec
        ig, ir = _ident(gpu["jpvt"], bid), _ident(ref["jpvt"], bid)
        off = 0
        for b in range(nb):
            w = int(ref["ncols"][b])
            assert set(ig[off:off + w]) == set(ir[off:off + w]), (prec, "block", b)
            off += w


@pytest.mark.gpu
def test_selection_stress_large_property(gpu_lib):
    """A larger case (2048 x 8192, 1024 bases, k = 1024) through the mixed
    path: the selection property and the backward error of the stopped
    factorisation (no oracle run at this size)."""
    import qrdm_gb300

    A0, bid = _case(2048, 8192, 1024, 7)
    gpu = qrdm_gb300.dgeqrdm(A0, nb=64, delta=0.9, tau_=0.15, precision="mixed", kstop=1024)
    _check_selection(A0, bid, gpu, 1024, "2048x8192 mixed")


@pytest.mark.gpu
def test_selection_stress_full_size_vs_reference(gpu_lib):
    """The 8192 x 32768 selection-stress matrix, stopped at k = 4096, against
    the compiled reference's pivots (tests/golden/selection32k_golden.npz,
    made by make_selection_golden.py): DM block sizes and per-block column
    identities over the blocks that reach k, both precisions, and the
    no-duplicate-base property."""
    import os

    import qrdm_gb300

    path = os.path.join(os.path.dirname(__file__), "golden", "selection32k_golden.npz")
    if not os.path.exists(path):
        pytest.skip("selection32k golden not generated")
    z = np.load(path)
    A0, bid = _case(8192, 32768, 4096, 5)
    assert np.array_equal(bid, z["bid"]), "regenerated matrix differs from the golden's"
    rng = np.random.default_rng(99)
    ri, ci = rng.integers(0, 8192, size=256), rng.integers(0, 32768, size=256)
    assert np.array_equal(A0[ri, ci], z["sample"]), "regenerated matrix differs from the golden's"
    kstop = 4096
    nbr, kr = _blocks(z["ncols"], kstop)
    ir = _ident(z["jpvt"], bid)
    for prec in ("mixed", "fp64"):
        gpu = qrdm_gb300.dgeqrdm(A0, nb=64, delta=0.9, tau_=0.15, precision=prec, kstop=kstop)
        assert gpu["info"] == 0
        nb, k = _blocks(gpu["ncols"], kstop)
        assert (nb, k) == (nbr, kr), (prec, nb, k, nbr, kr)
        assert np.array_equal(gpu["ncols"][:nb], z["ncols"][:nb]), prec
        ig = _ident(gpu["jpvt"], bid)
        off = 0
        for b in range(nb):
            w = int(z["ncols"][b])
            assert set(ig[off:off + w]) == set(ir[off:off + w]), (prec, "block", b)
            off += w
        sel = bid[gpu["jpvt"][:kstop] - 1]
        sel = sel[sel >= 0]
        assert len(np.unique(sel)) == len(sel)
