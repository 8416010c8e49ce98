"""Panel columns per grid barrier (QRDM_PANEL_GROUP = 1, 2, 4, 8).

The grouped panel (k_panel_grp) takes the partials of a group's later
columns from the exact totals of the group's start plus rank-one
corrections (a group ends early at a column that has lost more than 3/4 of
its square to the group's earlier reflectors); group 1 is the
one-column-per-barrier panel (k_panel_red).
Each setting runs in its own process (the library reads the variable once).
Bar: identical DM blocks and pivots wherever the oracle's decisions are
separated (Gaussian), leading R within 64 n eps ||A||_F of group 1's, and
the backward-error and orthogonality bounds in every case, including
panels whose columns lose almost all of their norm inside a group (the
group then ends early and the next starts from exact totals)."""
import os
import subprocess
import sys

import numpy as np
import pytest

EPS = 2.0 ** -53
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RUNNER = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import qrdm_gb300
from qrdm_gb300.QRDM import QRF
d = np.load(sys.argv[2])
A0 = np.asfortranarray(d["A"])
out = {}
if sys.argv[4] == "dgeqrf":
    A = A0.copy(order="F")
    tau = np.zeros(min(A.shape))
    out["info"] = np.array([QRF(102, A.shape[0], A.shape[1], A, A.shape[0], tau)])
    out["A"], out["tau"] = A, tau
else:
    r = qrdm_gb300.dgeqrdm(A0, nb=int(d["nb"]), tau_=float(d["tau_"]), precision=sys.argv[4])
    for k in ("A", "tau", "jpvt", "ncols"):
        out[k] = r[k]
    out["info"] = np.array([r["info"]])
np.savez(sys.argv[3], **out)
"""


def _run(tmp_path, A0, group, what, nb=64, tau_=0.15):
    inp = tmp_path / f"in_{group}_{what}_{nb}.npz"
    outp = tmp_path / f"out_{group}_{what}_{nb}.npz"
    np.savez(inp, A=A0, nb=np.int64(nb), tau_=np.float64(tau_))
    env = dict(os.environ, QRDM_PANEL_GROUP=str(group))
    subprocess.run([sys.executable, "-c", _RUNNER, ROOT, str(inp), str(outp), what], env=env,
                   check=True, timeout=600)
    d = np.load(outp)
    return {k: d[k] for k in d.files}


def _bounds(A0, r, pivoted=True):
    from qrdm_gb300.metrics import factor_metrics

    m, n = A0.shape
    jp = r["jpvt"] if pivoted else np.arange(1, n + 1, dtype=np.int32)
    met = factor_metrics(A0, r["A"], r["tau"], jp)
    assert met["backward"] <= 10 * max(m, n) * EPS, met
    assert met["orth"] <= 100 * max(m, n) * EPS, met
    return met


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_groups_agree_gaussian(gpu_lib, tmp_path, precision):
    from qrdm_gb300 import workloads as W

    A0 = W.gaussian(3000, 2000, seed=71)
    runs = {g: _run(tmp_path, A0, g, precision) for g in (1, 2, 4, 8)}
    base = runs[1]
    an = np.linalg.norm(A0)
    for g, r in runs.items():
        assert int(r["info"][0]) == 0
        assert np.array_equal(r["ncols"], base["ncols"]), g
        assert np.array_equal(r["jpvt"], base["jpvt"]), g
        dR = np.linalg.norm(np.triu(r["A"][:2000]) - np.triu(base["A"][:2000]))
        assert dR <= 64 * 2000 * EPS * an, (g, dR / an)
        _bounds(A0, r)


@pytest.mark.gpu
def test_groups_dependent_columns(gpu_lib, tmp_path):
    """Rank 300 plus 1e-10 noise: inside DM blocks the candidates lose most
    of their norm to earlier columns, the case the early group end guards."""
    from qrdm_gb300 import workloads as W

    A0 = W.low_rank_noise(2000, 1200, 300, 1e-10, seed=72)
    for g in (1, 4, 8):
        r = _run(tmp_path, A0, g, "fp64")
        assert int(r["info"][0]) == 0
        _bounds(A0, r)
        d = np.abs(np.diag(r["A"][:1200, :1200]))
        assert d[299] / d[0] > 1e-3 and d[300] / d[0] < 1e-7, (g, d[299] / d[0], d[300] / d[0])


@pytest.mark.gpu
def test_groups_unpivoted_rank_deficient(gpu_lib, tmp_path):
    """Plain dgeqrf (no early exit) on columns that repeat earlier ones up
    to 1e-12: the corrected norms would cancel; the group ends early and
    the reflectors stay orthogonal."""
    rng = np.random.default_rng(73)
    m, n = 1500, 256
    B = rng.standard_normal((m, 40))
    A0 = np.asfortranarray(B @ rng.standard_normal((40, n)) + 1e-12 * rng.standard_normal((m, n)))
    for g in (1, 4, 8):
        r = _run(tmp_path, A0, g, "dgeqrf")
        assert int(r["info"][0]) == 0
        _bounds(A0, r, pivoted=False)


@pytest.mark.gpu
def test_groups_block_width_128(gpu_lib, tmp_path):
    """DM blocks of up to 128 columns (the widest the device path takes):
    the grouped panel's slabs and totals at their largest."""
    from qrdm_gb300 import workloads as W

    A0 = W.gaussian(3000, 1500, seed=74)
    base = _run(tmp_path, A0, 1, "mixed", nb=128)
    an = np.linalg.norm(A0)
    for g in (1, 4):
        r = base if g == 1 else _run(tmp_path, A0, g, "mixed", nb=128)
        assert int(r["info"][0]) == 0
        assert np.array_equal(r["ncols"], base["ncols"]) and np.array_equal(r["jpvt"], base["jpvt"]), g
        dR = np.linalg.norm(np.triu(r["A"][:1500]) - np.triu(base["A"][:1500]))
        assert dR <= 64 * 1500 * EPS * an, (g, dR / an)
        _bounds(A0, r)


@pytest.mark.gpu
def test_groups_no_early_exit_graded(gpu_lib, tmp_path):
    """tau_ = 0 (no early exit) on 1200 x 1200 with singular values down to
    1e-12: inside a panel columns lose most of their norm, so groups end
    early, and the factorisation stays within the bounds for every group
    size."""
    from qrdm_gb300 import workloads as W

    A0 = W.graded_svd(1200, seed=75)
    for g in (1, 4, 8):
        r = _run(tmp_path, A0, g, "fp64", tau_=0.0)
        assert int(r["info"][0]) == 0
        _bounds(A0, r)
