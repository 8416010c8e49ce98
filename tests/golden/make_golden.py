"""Generates tests/golden/dmqr_golden.npz and qp3_golden.npz by running the
compiled, unmodified reference (oracle/_ref/libqrdm_ref.so, built from the
mdessole/qrdm sources by oracle/build_ref.sh) on small seeded inputs.

The reference ships no test vectors (its only exercise is an unseeded
notebook), so these fixtures are the known answers that pin both the CPU
oracle and the GPU library.  Inputs are stored with the outputs, so the
fixtures do not depend on the generator's floating-point reproducibility.

Run where the reference sources are present, naming their root:
    QRDM_REFERENCE_ROOT=<reference root> OPENBLAS_NUM_THREADS=1 python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference, build_reference  # noqa: E402
from qrdm_gb300 import workloads as W  # noqa: E402


def cases():
    """(name, input_key, params); params = dict(delta, tau_, nb, stop, eta)."""
    d = dict(delta=0.9, tau_=0.15, nb=64, stop=0, eta=0.0)
    rng = np.random.default_rng(11)
    inputs = {}
    inputs["demo128"] = W.rank_deficient_demo(128, seed=7)
    inputs["graded160"] = W.graded_svd(160, seed=0)
    inputs["tall160x96"] = W.gaussian(160, 96, seed=21)
    inputs["wide64x150"] = W.gaussian(64, 150, seed=22)
    inputs["kahan128"] = W.kahan(128, seed=23)
    inputs["kahan96"] = W.kahan(96, seed=24)
    a = W.gaussian(100, 80, seed=25)
    a[:, ::8] = 0.0
    inputs["zerocols100x80"] = a
    base = W.gaussian(120, 30, seed=26)
    inputs["dupcols120x90"] = np.asfortranarray(base[:, rng.integers(0, 30, size=90)])
    inputs["gauss60x50"] = W.gaussian(60, 50, seed=27)
    inputs["gauss50x40"] = W.gaussian(50, 40, seed=28)
    inputs["gauss80x60"] = W.gaussian(80, 60, seed=29)
    inputs["graded80"] = W.graded_svd(80, seed=30)
    inputs["row1x7"] = W.gaussian(1, 7, seed=33)
    inputs["col7x1"] = W.gaussian(7, 1, seed=34)
    inputs["one1x1"] = W.gaussian(1, 1, seed=35)
    inputs["two2x2"] = W.gaussian(2, 2, seed=36)
    inputs["tiny64"] = W.gaussian(64, 64, seed=37) * 1e-160
    inputs["huge64"] = W.gaussian(64, 64, seed=38) * 1e150
    inputs["lowrank160x96"] = W.low_rank_noise(160, 96, 24, 1e-10, seed=39)
    inputs["select96x256"] = W.selection_stress(96, 256, 48, seed=40)
    out = [
        ("demo128", "demo128", d),
        ("demo128_stop1", "demo128", {**d, "stop": 1}),
        ("demo128_stop2", "demo128", {**d, "stop": 2}),
        ("demo128_stop3", "demo128", {**d, "stop": 3, "eta": 1e-9}),
        ("graded160", "graded160", d),
        ("graded160_nb16", "graded160", {**d, "nb": 16}),
        ("tall160x96_nb16", "tall160x96", {**d, "nb": 16}),
        ("wide64x150_nb32", "wide64x150", {**d, "nb": 32}),
        ("kahan128", "kahan128", d),
        ("kahan96_nb8", "kahan96", {**d, "nb": 8}),
        ("zerocols100x80", "zerocols100x80", d),
        ("dupcols120x90", "dupcols120x90", d),
        ("nb1_gauss60x50", "gauss60x50", {**d, "nb": 1}),
        ("nbbig_gauss50x40", "gauss50x40", d),
        ("delta0_gauss80x60", "gauss80x60", {**d, "delta": 0.0}),
        ("tau1_gauss80x60", "gauss80x60", {**d, "tau_": 1.0}),
        ("delta1_graded80", "graded80", {**d, "delta": 1.0}),
        ("tau0_graded80", "graded80", {**d, "tau_": 0.0}),
        ("row1x7", "row1x7", d),
        ("col7x1", "col7x1", d),
        ("one1x1", "one1x1", d),
        ("two2x2", "two2x2", d),
        ("tiny64", "tiny64", d),
        ("huge64", "huge64", d),
        ("lowrank160x96", "lowrank160x96", d),
        ("lowrank160x96_stop3", "lowrank160x96", {**d, "stop": 3, "eta": 1e-8}),
        ("select96x256_nb32", "select96x256", {**d, "nb": 32}),
    ]
    return inputs, out


def main():
    build_reference()
    ref = Reference()
    store = {}
    names = []
    inputs, plan = cases()
    for key, A0 in inputs.items():
        store[f"in/{key}"] = np.asfortranarray(A0)
    for name, key, p in plan:
        A0 = inputs[key]
        A = np.array(A0, dtype=np.float64, order="F", copy=True)
        m, n = A.shape
        jpvt = np.zeros(n, np.int32)
        tau = np.zeros(min(m, n), np.float64)
        ncols = np.zeros(n, np.int32)
        ncols[0] = p["stop"]
        thres = np.array([p["delta"], p["tau_"], p["eta"]], np.float64)
        info = ref.dgeqrdm(102, m, n, A, m, jpvt, tau, ncols, thres, p["nb"])
        names.append(name)
        store[f"{name}/input"] = np.array([key])
        store[f"{name}/params"] = np.array([p["delta"], p["tau_"], p["nb"], p["stop"], p["eta"]])
        store[f"{name}/info"] = np.array([info])
        store[f"{name}/A_out"] = A
        store[f"{name}/jpvt"] = jpvt
        store[f"{name}/tau"] = tau
        store[f"{name}/ncols"] = ncols
        print(f"{name:24s} {m}x{n} info={info} ncols={ncols[:8].tolist()}")
    store["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "dmqr_golden.npz"), **store)

    # QP3: the reference's dgeqp3 wrapper (src/dgeqp3.c) over LAPACK 3.12
    q = {}
    qn = []
    for name, A0 in [("gauss90x70", W.gaussian(90, 70, seed=50)),
                     ("graded100", W.graded_svd(100, seed=51)),
                     ("wide40x100", W.gaussian(40, 100, seed=52)),
                     ("kahan80", W.kahan(80, seed=53))]:
        A = np.array(A0, order="F", copy=True)
        m, n = A.shape
        jpvt = np.zeros(n, np.int32)
        tau = np.zeros(min(m, n))
        info = ref.dgeqp3(102, m, n, A, m, jpvt, tau)
        qn.append(name)
        q[f"{name}/A_in"] = np.asfortranarray(A0)
        q[f"{name}/A_out"] = A
        q[f"{name}/jpvt"] = jpvt
        q[f"{name}/tau"] = tau
        q[f"{name}/info"] = np.array([info])
        print(f"qp3 {name:16s} info={info} jpvt[:8]={jpvt[:8].tolist()}")
    q["names"] = np.array(qn)
    np.savez_compressed(os.path.join(HERE, "qp3_golden.npz"), **q)


if __name__ == "__main__":
    main()
