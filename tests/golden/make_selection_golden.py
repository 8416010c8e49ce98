"""Generates tests/golden/selection32k_golden.npz: the compiled, unmodified
reference (oracle/_ref/libqrdm_ref.so, see oracle/build_ref.sh) run on the
8192 x 32768 column-subset-selection stress matrix
(qrdm_gb300.workloads.selection_stress(8192, 32768, 4096, seed=5): 4096
N(0,1) base columns repeated U{1..8} times with a 1e-8 relative
perturbation, N(0,1) 10^-U[0,6] fillers, shuffled), delta = 0.9,
tau_ = 0.15, nb = 64, full factorisation.

The 2 GB input is not stored: it is regenerated from its seed (NumPy's
PCG64 streams are platform independent), and the fixture keeps the base
index of every column plus a seeded sample of entries to check that the
regenerated matrix is the one the reference saw.

Run after the compiled reference exists (oracle/build_ref.sh, or
__graft_entry__.build() where the reference sources are present):
    python tests/golden/make_selection_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference, run_dmqr  # noqa: E402
from qrdm_gb300 import workloads as W  # noqa: E402

M, N, NBASE, SEED = 8192, 32768, 4096, 5


def sample_index(m, n, count=256, seed=99):
    rng = np.random.default_rng(seed)
    return rng.integers(0, m, size=count), rng.integers(0, n, size=count)


def main():
    A, bid = W.selection_stress(M, N, NBASE, seed=SEED, return_base=True)
    ri, ci = sample_index(M, N)
    sample = A[ri, ci].copy()
    r = run_dmqr(Reference(), A, delta=0.9, tau_=0.15, nb=64)
    np.savez_compressed(os.path.join(HERE, "selection32k_golden.npz"), jpvt=r["jpvt"].astype(np.int32),
                        ncols=r["ncols"].astype(np.int32), bid=bid.astype(np.int32), sample=sample,
                        info=np.array([r["info"]], np.int32))
    print("info", r["info"], "blocks", int(np.count_nonzero(r["ncols"])))


if __name__ == "__main__":
    main()
