"""Seeded synthetic inputs for the DM-QR workloads.

None of the workloads comes from a public benchmark suite; they are the
matrix families the DM-QR benchmark configurations describe, generated with
NumPy's PCG64 ``default_rng`` so that every run sees the same matrices.
All matrices are float64 and returned in Fortran (column-major) order, the
layout the ``dgeqrdm`` entry point expects (LAPACK_COL_MAJOR = 102).

Flop counts used for "effective FP64 TFLOP/s":
  full factorisation      F = 2 m n^2 - 2 n^3 / 3            (m >= n)
  stop after k columns    F = 4 m n k - 2 (m + n) k^2 + 4 k^3 / 3
"""
from __future__ import annotations

import math

import numpy as np


def flops_full(m: int, n: int) -> float:
    """Householder QR flop count (LAPACK convention, m >= n; else swap)."""
    if m >= n:
        return 2.0 * m * n * n - 2.0 * n ** 3 / 3.0
    return 2.0 * n * m * m - 2.0 * m ** 3 / 3.0


def flops_k(m: int, n: int, k: int) -> float:
    """Flops of a QR that stops after k columns (k <= min(m, n))."""
    return 4.0 * m * n * k - 2.0 * (m + n) * k * k + 4.0 * k ** 3 / 3.0


def _orth(rng, m, n):
    q, _ = np.linalg.qr(rng.standard_normal((m, n)))
    return q


def graded_svd(n: int = 1000, seed: int = 0, decades: float = 12.0) -> np.ndarray:
    """A = U diag(s) V^T, U, V orthogonal factors of seeded N(0,1) n x n
    matrices, s_i = 10^(-decades (i-1)/(n-1)).  (DM-QR CPU parity workload,
    1000 x 1000 with 12 decades.)"""
    rng = np.random.default_rng(seed)
    u = _orth(rng, n, n)
    v = _orth(rng, n, n)
    s = 10.0 ** (-decades * np.arange(n) / max(n - 1, 1))
    return np.asfortranarray((u * s) @ v.T)


def gaussian(m: int, n: int, seed: int = 1) -> np.ndarray:
    """i.i.d. N(0,1) entries."""
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal((m, n)))


def kahan(n: int = 4096, c: float = 0.285, noise: float = 1e-14, seed: int = 2) -> np.ndarray:
    """Kahan matrix diag(s^(i-1)) (I - c * strict_upper_ones), s = sqrt(1-c^2),
    plus a seeded noise * N(0,1) perturbation (stresses pivot ties and norm
    downdating)."""
    s = math.sqrt(1.0 - c * c)
    k = np.triu(-c * np.ones((n, n)), 1) + np.eye(n)
    k *= (s ** np.arange(n))[:, None]
    rng = np.random.default_rng(seed)
    return np.asfortranarray(k + noise * rng.standard_normal((n, n)))


def low_rank_noise(m: int = 16384, n: int = 8192, r: int = 2048, noise: float = 1e-10,
                   seed: int = 3) -> np.ndarray:
    """A = L R^T + noise * E with L (m x r), R (n x r) i.i.d. N(0,1)/sqrt(r) and
    E i.i.d. N(0,1): numerical rank r.  (Mixed-precision DM-QR workload,
    16384 x 8192, rank 2048.)"""
    rng = np.random.default_rng(seed)
    lf = rng.standard_normal((m, r)) / math.sqrt(r)
    rf = rng.standard_normal((n, r)) / math.sqrt(r)
    a = np.asfortranarray(lf @ rf.T)
    a += noise * rng.standard_normal((m, n))
    return a


def selection_stress(m: int = 8192, n: int = 32768, nbase: int = 4096, seed: int = 5,
                     rel: float = 1e-8, return_base: bool = False):
    """Column-subset-selection stress matrix: nbase N(0,1) base columns, each
    repeated U{1..8} times with a (1 + rel * N(0,1)) entrywise perturbation,
    the rest N(0,1) * 10^(-u), u ~ U[0,6]; truncated/filled to n columns and
    shuffled by seed.  return_base: also the base index of every column
    (-1 for the filler columns)."""
    rng = np.random.default_rng(seed)
    base = rng.standard_normal((m, nbase))
    reps = rng.integers(1, 9, size=nbase)
    cols = []
    total = 0
    for j in range(nbase):
        for _ in range(int(reps[j])):
            if total >= n:
                break
            cols.append((j, True))
            total += 1
    a = np.empty((m, n), order="F")
    for t, (j, _) in enumerate(cols):
        a[:, t] = base[:, j] * (1.0 + rel * rng.standard_normal(m))
    for t in range(len(cols), n):
        u = rng.uniform(0.0, 6.0)
        a[:, t] = rng.standard_normal(m) * 10.0 ** (-u)
    perm = rng.permutation(n)
    if return_base:
        bid = np.full(n, -1, np.int64)
        bid[:len(cols)] = [j for j, _ in cols]
        return np.asfortranarray(a[:, perm]), bid[perm]
    return np.asfortranarray(a[:, perm])


def batched_shapes(count: int = 2000, seed: int = 4, nmin: int = 32, nmax: int = 512,
                   rmax: float = 4.0, mcap: int = 2048):
    """Shapes of the uneven batched workload: n log-uniform in [nmin, nmax],
    m = min(ceil(n r), mcap) with r log-uniform in [1, rmax]."""
    rng = np.random.default_rng([seed, 0])
    n = np.exp(rng.uniform(math.log(nmin), math.log(nmax), size=count)).astype(int)
    r = np.exp(rng.uniform(0.0, math.log(rmax), size=count))
    m = np.minimum(np.ceil(n * r).astype(int), mcap)
    m = np.maximum(m, n)
    return m.astype(np.int64), n.astype(np.int64)


def batched_matrix(i: int, m: int, n: int, seed: int = 4) -> np.ndarray:
    """Matrix i of the batched workload: U diag(s) V^T with U (m x n), V (n x n)
    orthonormal from seeded Gaussians and s geometric from 1 to 10^(-d),
    d ~ U[4, 14]."""
    rng = np.random.default_rng([seed, int(i) + 1])
    d = rng.uniform(4.0, 14.0)
    u = _orth(rng, m, n)
    v = _orth(rng, n, n)
    s = 10.0 ** (-d * np.arange(n) / max(n - 1, 1))
    return np.asfortranarray((u * s) @ v.T)


def rank_deficient_demo(n: int = 128, seed: int = 7) -> np.ndarray:
    """The notebook-style matrix (seeded): singular values 2^(1-i) + 1e-17 with
    a bump on the first n/2 (numerical rank n/2)."""
    rng = np.random.default_rng(seed)
    u = _orth(rng, n, n)
    v = _orth(rng, n, n)
    r = n // 2
    sv = np.exp2(1.0 - np.arange(1, n + 1)) + 1e-17
    sv[:r] += 0.01 * (r - np.arange(1, r + 1))
    return np.asfortranarray((u * sv) @ v.T)
