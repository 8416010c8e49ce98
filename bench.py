"""Benchmark of the GB300 DM-QR hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload lowrank16k|gauss4k|kahan4k|graded1k|batched2000]
                    [--precision mixed|fp64] [--no-variants]

One step = one DM-QR factorisation of the workload matrix, already resident
in HBM (restored from a pristine device copy before each step; the copy is
inside the timed region).  The default workload is the 16384 x 8192
numerical-rank-2048 matrix A = L R^T + 1e-10 E (full factorisation, nb = 64,
delta = 0.9, tau_ = 0.15) in the mixed-precision form (Ozaki-split FP16
trailing update, BF16 cosine Gram with FP64 recheck).  Inputs (1.07 GB) are
larger than the 129 MB L2, so no explicit flush is needed between steps.

--workload batched2000: one step = the batched DM-QR of 2000 uneven
matrices (n log-uniform in [32, 512], m = n r, r log-uniform in [1, 4],
capped at 2048; U diag(s) V^T with geometric decay to 10^-d, d ~ U[4, 14])
in one persistent launch; value = matrices/s; the roofline is the summed
per-problem bound sum_i max(F_i / P_fp64, 16 m_i n_i / BW).

value = effective FP64 TFLOP/s = F / t with F = 2 m n^2 - 2 n^3 / 3 (whole job
over all ranks; ranks run independent replicas).  e2e = the same metric
through the host C ABI (dgeqrdm_ex: pinned host buffers, H2D + factorisation
+ D2H inside the timed call).  --impl reference times the CPU restatement of
the reference (oracle/, OpenBLAS on all host threads) on a bounded sample of
the same workload: the factorisation of the same matrix stopped after 2048
columns (F = 4 m n k - 2 (m + n) k^2 + 4 k^3 / 3).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (m, n, description)
    "lowrank16k": (16384, 8192, "A = L R^T + 1e-10 E, L 16384x2048, R 8192x2048 N(0,1)/sqrt(2048)"),
    "gauss4k": (4096, 4096, "i.i.d. N(0,1)"),
    "kahan4k": (4096, 4096, "Kahan c=0.285 + 1e-14 N(0,1)"),
    "graded1k": (1000, 1000, "U diag(10^(-12(i-1)/999)) V^T"),
    "batched2000": (0, 0, "2000 uneven U diag(s) V^T, n in [32, 512], m = n r, r in [1, 4]"),
    "select32k": (8192, 32768, "selection stress: 4096 N(0,1) base columns repeated U{1..8} times "
                               "(1e-8 relative perturbation), filler N(0,1) 10^-U[0,6], shuffled"),
}
KSTOP = {"select32k": 4096}  # column-subset selection: stop after k columns
SELECTION_BASES = {}
BATCH_COUNT, BATCH_NB = 2000, 32
BATCH_GENERATOR = None
BATCH_CPU_SAMPLE = 400
FP64_RATES = None
NB, DELTA, TAU_ = 64, 0.9, 0.15
CPU_SAMPLE_K = 2048


def flops_full(m, n):
    return 2.0 * m * n * n - 2.0 * n ** 3 / 3.0 if m >= n else 2.0 * n * m * m - 2.0 * m ** 3 / 3.0


def flops_k(m, n, k):
    return 4.0 * m * n * k - 2.0 * (m + n) * k * k + 4.0 * k ** 3 / 3.0


def make_matrix_device(name, seed=3):
    """Column-major workload matrix as a float64 tensor of shape (n, m) on
    the GPU (on the CPU where no GPU exists: the multi-process tests of the
    reference arm; the low-rank matrix then comes from the CPU generator)."""
    import torch

    m, n, _ = WORKLOADS[name]
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    g = torch.Generator(device=dev).manual_seed(seed)
    if name == "lowrank16k":
        r = 2048
        lf = torch.randn(m, r, generator=g, dtype=torch.float64, device=dev) / math.sqrt(r)
        rf = torch.randn(n, r, generator=g, dtype=torch.float64, device=dev) / math.sqrt(r)
        at = rf @ lf.T
        at += 1e-10 * torch.randn(n, m, generator=g, dtype=torch.float64, device=dev)
        return at.contiguous()
    if name == "select32k":
        from qrdm_gb300 import workloads as W

        a, bid = W.selection_stress(m, n, 4096, seed=5, return_base=True)
        SELECTION_BASES[name] = bid
        return torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)
    from qrdm_gb300 import workloads as W

    if name == "gauss4k":
        a = W.gaussian(m, n, seed=1)
    elif name == "kahan4k":
        a = W.kahan(n, seed=2)
    else:
        a = W.graded_svd(n, seed=0)
    return torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p is not None:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()
                self.out = ""

    def summary(self):
        rows = []
        for line in (self.out or "").strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows)}


def dist_setup(n_gpus):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:  # host-only ranks (the tests of the multi-process path)
            dist.init_process_group("gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def fp64_rates():
    """Measured FP64 rates of this GPU in TFLOP/s (the library's
    qrdm_fp64_rates: independent FMA chains on the CUDA cores, FP64
    tensor-core MMAs at two shapes), measured once per process."""
    global FP64_RATES
    if FP64_RATES is None:
        from qrdm_gb300 import lib

        out = (C.c_double * 3)()
        rc = lib().qrdm_fp64_rates(out, 3)
        FP64_RATES = ({"fma": out[0], "dmma_m8n8k4": out[1], "dmma_m16n8k16": out[2]}
                      if rc == 0 else {})
    return FP64_RATES


def legacy_mma_rates():
    """Rates of the warp-level tensor-core MMA (the library's
    qrdm_legacy_mma_rates): INT8 in TOP/s and FP16 in TFLOP/s.  This GPU's
    tcgen05 MMA has no INT8 kind, so the INT8 figure bounds what INT8 digits
    (exact INT32 accumulation) could reach against the FP16 digits the Ozaki
    split runs on tcgen05."""
    from qrdm_gb300 import lib

    out = (C.c_double * 2)()
    rc = lib().qrdm_legacy_mma_rates(out, 2)
    if rc != 0:
        return {}
    return {"int8_mma_sync_tops": out[0], "fp16_mma_sync_tflops": out[1],
            "tcgen05_kind_i8": "not accepted by the assembler for sm_103a"}


def fp64_peak():
    """(TFLOP/s, description) of the FP64 roof: the best measured FP64 rate."""
    r = fp64_rates()
    if r:
        best = max(r, key=r.get)
        return r[best], f"measured ({best}, qrdm_fp64_rates: best of the FMA and FP64 MMA kernels)"
    return 1.25, "nominal (the FP64 rate measurement failed)"


def load_traffic(kernel_key):
    """Per-launch DRAM traffic of a kernel from a committed ncu summary
    (profiles/traffic.txt lines: '<key> <bytes_per_unit> <unit>'), or None."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel_key:
                try:
                    return float(parts[1])
                except ValueError:
                    return None
    return None


def cpu_sample(name, threads, at_host=None, margins=False):
    """Oracle (CPU restatement of the reference, OpenBLAS) on the bounded
    sample: the workload matrix factored until >= CPU_SAMPLE_K columns.
    margins=True also records every decision's margin (the oracle's run is
    then the parity check of the GPU factorisation of the same matrix)."""
    from oracle.oracle import Oracle, run_dmqr

    m, n, _ = WORKLOADS[name]
    if at_host is None:
        at_host = make_matrix_device(name).cpu().numpy()
    A0 = at_host.T  # Fortran-ordered m x n view
    o = Oracle(threads=threads)
    k_target = min(CPU_SAMPLE_K, min(m, n))
    t0 = time.perf_counter()
    r = run_dmqr(o, A0, nb=NB, delta=DELTA, tau_=TAU_, kstop=k_target, margins=margins)
    dt = time.perf_counter() - t0
    k = int(np.sum(r["ncols"]))
    f = flops_k(m, n, k) if k < min(m, n) else flops_full(m, n)
    return {"value": f / dt / 1e12, "seconds": dt, "k": k, "flops": f, "run": r}


def parity_vs_oracle(ref, gpu_jpvt, gpu_ncols, gpu_rdiag, gap=100.0):
    """The GPU factorisation against the oracle's run of the same matrix
    (bit-identical to the compiled reference): jpvt and DM block sizes over
    the oracle's gap-separated prefix (every decision >= gap noise units from
    its threshold), how far they agree beyond it, and the |R_kk| profile over
    the columns the oracle factored."""
    from oracle.oracle import separated_prefix

    pb, pc = separated_prefix(ref, gap)
    rj, rn = ref["jpvt"], ref["ncols"]
    kref = int(np.sum(rn))
    nblk = int(np.count_nonzero(rn))
    same_blocks = bool(np.array_equal(gpu_ncols[:pb], rn[:pb]))
    identical = bool(same_blocks and np.array_equal(gpu_jpvt[:pc], rj[:pc]))
    # leading columns where the two runs made the same choices
    agree_cols = 0
    cols = 0
    for b in range(nblk):
        if gpu_ncols[b] != rn[b] or not np.array_equal(gpu_jpvt[cols:cols + rn[b]], rj[cols:cols + rn[b]]):
            break
        cols += int(rn[b])
        agree_cols = cols
    rd_ref = np.abs(np.diag(ref["A"])[:kref])
    rd_gpu = np.abs(np.asarray(gpu_rdiag)[:kref])
    ratio = np.where(rd_ref > 0, rd_gpu / np.where(rd_ref > 0, rd_ref, 1.0), 1.0)
    pre = ratio[:pc] if pc > 0 else ratio[:0]
    return {"gap_noise_units": gap, "prefix_blocks": int(pb), "prefix_cols": int(pc),
            "identical": identical, "agree_cols": int(agree_cols),
            "agree_cols_beyond_prefix": int(max(0, agree_cols - pc)),
            "oracle_cols": kref, "oracle_blocks": nblk,
            "rkk_ratio_max_dev_prefix": float(np.max(np.abs(pre - 1.0))) if pre.size else None,
            "rkk_ratio_max_dev_all": float(np.max(np.abs(ratio - 1.0))) if ratio.size else None,
            "rkk_ratio_median_dev_all": float(np.median(np.abs(ratio - 1.0))) if ratio.size else None}


def run_reference(args):
    import torch

    rank, world, _ = dist_setup(args.gpus)
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    at = make_matrix_device(args.workload).cpu().numpy()
    m, n, desc = WORKLOADS[args.workload]
    for _ in range(args.warmup):
        cpu_sample(args.workload, threads, at)
    vals, secs = [], []
    for _ in range(args.steps):
        s = cpu_sample(args.workload, threads, at)
        vals.append(s["value"])
        secs.append(s["seconds"])
    v = statistics.median(vals)
    sample = (f"{args.workload} {m}x{n} factored until >= {CPU_SAMPLE_K} columns "
              f"(k={s['k']}), oracle port of the reference on OpenBLAS")
    # the whole factorisation of the same matrix, once, so the sample's rate
    # can be compared with the full run's (the GPU arm's unit of work)
    full = None
    if args.full_run:
        from oracle.oracle import Oracle, run_dmqr

        o = Oracle(threads=threads)
        t0 = time.perf_counter()
        r = run_dmqr(o, at.T, nb=NB, delta=DELTA, tau_=TAU_, kstop=KSTOP.get(args.workload, 0))
        dt = time.perf_counter() - t0
        kf = int(np.sum(r["ncols"]))
        ff = flops_k(m, n, kf) if kf < min(m, n) else flops_full(m, n)
        full = {"seconds": dt, "tflops": ff / dt / 1e12, "columns": kf, "info": int(r["info"]),
                "note": "one untimed-loop run of the whole factorisation of the same matrix"}
    line = {"impl": "reference", "metric": "DM-QR effective FP64 TFLOP/s", "value": v,
            "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.median(secs) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "m": m, "n": n, "nb": NB, "delta": DELTA,
                       "tau_": TAU_, "matrix": desc, "sample_columns": s["k"]},
            "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "full_run": full}
    print(json.dumps(line), flush=True)


def device_backward(L, work, tau, jp, pristine, m, n, k):
    """||A P - Q R||_F / ||A||_F of a device-resident factorisation (Q R
    formed by the library's DORMQR applied to R)."""
    import torch

    Af = work.T
    R = torch.zeros_like(Af)
    R[:k, :] = torch.triu(Af[:k, :])
    if k < min(m, n):
        R[k:, k:] = Af[k:, k:]
    QR = R.T.contiguous()
    del R
    rq = L.qrdm_dormqr_dev(102, m, n, k, C.c_void_p(work.data_ptr()), m, C.c_void_p(tau.data_ptr()),
                           C.c_void_p(QR.data_ptr()), m)
    if rq != 0:
        return None
    be = float(torch.linalg.norm(QR - pristine[jp.long() - 1]) / torch.linalg.norm(pristine))
    del QR
    return be


def single_config(L, stream, name, precisions=("fp64", "mixed"), qp3=False):
    """One workload of the other configurations, device-resident: one
    untimed call (workspace growth), then one factorisation per precision
    timed with CUDA events on the library's stream; backward error of each;
    the GPU QP3 comparator on the same matrix when asked."""
    import qrdm_gb300
    import torch

    from qrdm_gb300 import Stats, default_options

    m, n, desc = WORKLOADS[name]
    kstop = KSTOP.get(name, 0)
    pristine = make_matrix_device(name)
    work = torch.empty_like(pristine)
    jp = torch.zeros(n, dtype=torch.int32, device="cuda")
    tau = torch.zeros(min(m, n), dtype=torch.float64, device="cuda")
    thres = np.array([DELTA, TAU_, 0.0])
    pd = C.POINTER(C.c_double)
    out = {"m": m, "n": n, "matrix": desc, "kstop": kstop}

    def run(prec):
        work.copy_(pristine)
        jp.zero_()
        nc = np.zeros(n, np.int32)
        opt = default_options(precision=qrdm_gb300.PREC[prec], kstop=kstop)
        st = Stats()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        info = L.dgeqrdm_dev(102, m, n, C.c_void_p(work.data_ptr()), m, C.c_void_p(jp.data_ptr()),
                             C.c_void_p(tau.data_ptr()), nc.ctypes.data_as(C.POINTER(C.c_int)),
                             thres.ctypes.data_as(pd), NB, C.byref(opt), C.byref(st))
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), nc, info, st

    for prec in precisions:
        run(prec)
        ms, nc, info, st = run(prec)
        if info != 0:
            out[prec] = {"info": int(info)}
            continue
        k = int(np.sum(nc))
        F = flops_k(m, n, k) if k < min(m, n) else flops_full(m, n)
        r = {"ms": ms, "tflops": F / (ms / 1e3) / 1e12, "blocks": int(np.count_nonzero(nc)),
             "columns": k, "launches": int(st.launches)}
        if name in SELECTION_BASES:
            bid = SELECTION_BASES[name]
            sel = bid[jp[:kstop].cpu().numpy().astype(np.int64) - 1]
            sel = sel[sel >= 0]
            r["selected_bases"] = int(len(sel))
            r["distinct_bases"] = bool(len(np.unique(sel)) == len(sel))
        r["backward"] = device_backward(L, work, tau, jp, pristine, m, n, min(k, m, n))
        out[prec] = r
    if qp3:
        work.copy_(pristine)
        jp.zero_()
        q0 = torch.cuda.Event(enable_timing=True)
        q1 = torch.cuda.Event(enable_timing=True)
        q0.record(stream)
        rq = L.dgeqp3_dev(102, m, n, C.c_void_p(work.data_ptr()), m, C.c_void_p(jp.data_ptr()),
                          C.c_void_p(tau.data_ptr()))
        q1.record(stream)
        torch.cuda.synchronize()
        if rq == 0:
            qms = q0.elapsed_time(q1)
            out["qp3"] = {"ms": qms, "tflops": flops_full(m, n) / (qms / 1e3) / 1e12,
                          "backward": device_backward(L, work, tau, jp, pristine, m, n, min(m, n))}
            if "fp64" in out and "ms" in out["fp64"]:
                out["fp64_dmqr_over_qp3_speedup"] = qms / out["fp64"]["ms"]
            if "mixed" in out and "ms" in out["mixed"]:
                out["mixed_dmqr_over_qp3_speedup"] = qms / out["mixed"]["ms"]
    if "fp64" in out and "mixed" in out and "ms" in out["fp64"] and "ms" in out["mixed"]:
        out["mixed_over_fp64_speedup"] = out["fp64"]["ms"] / out["mixed"]["ms"]
    del pristine, work
    torch.cuda.empty_cache()
    return out


def other_configs(L, stream):
    """The other benchmark configurations, one measured step each, for the
    default run's line: FP64 DM-QR vs QP3 on the 4096^2 Gaussian and Kahan
    matrices (mixed beside them), the 8192 x 32768 selection stress stopped
    at 4096 columns, and the 2000-matrix batched launch."""
    res = {}
    for name in ("gauss4k", "kahan4k"):
        try:
            res[name] = single_config(L, stream, name, qp3=True)
        except Exception as exc:
            res[name] = {"error": str(exc)[:200]}
    try:
        res["select32k"] = single_config(L, stream, "select32k", precisions=("mixed",))
    except Exception as exc:
        res["select32k"] = {"error": str(exc)[:200]}
    try:
        bm = batched_measure(L, stream, steps=1, warmup=1)
        res["batched2000"] = {"matrices_per_s": bm["value"], "ms": bm["ms"], "kernel_ms": bm["kernel_ms"],
                              "nb": bm["nb"], "precision": bm["precision"], "e2e": bm["e2e"],
                              "roofline": bm["roofline"], "errors": bm["errors"],
                              "phase_share": bm["phase_share"]}
    except Exception as exc:
        res["batched2000"] = {"error": str(exc)[:200]}
    return res


def run_ours(args):
    import torch

    import qrdm_gb300
    from qrdm_gb300 import Stats, default_options, lib

    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    L = lib()
    m, n, desc = WORKLOADS[args.workload]
    prec = qrdm_gb300.PREC[args.precision]
    stream = torch.cuda.current_stream()
    L.qrdm_set_stream(C.c_void_p(stream.cuda_stream))
    pristine = make_matrix_device(args.workload)
    work = torch.empty_like(pristine)
    jp = torch.zeros(n, dtype=torch.int32, device="cuda")
    tau = torch.zeros(min(m, n), dtype=torch.float64, device="cuda")
    thres = np.array([DELTA, TAU_, 0.0])
    pd = C.POINTER(C.c_double)

    def step(stats=None, precision=prec):
        work.copy_(pristine)
        jp.zero_()
        nc = np.zeros(n, np.int32)
        opt = default_options(precision=precision, kstop=KSTOP.get(args.workload, 0), slices=args.slices)
        st = stats if stats is not None else Stats()
        info = L.dgeqrdm_dev(102, m, n, C.c_void_p(work.data_ptr()), m, C.c_void_p(jp.data_ptr()),
                             C.c_void_p(tau.data_ptr()), nc.ctypes.data_as(C.POINTER(C.c_int)),
                             thres.ctypes.data_as(pd), NB, C.byref(opt), C.byref(st))
        if info != 0:
            raise RuntimeError(f"dgeqrdm_dev info={info}")
        return st, nc

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    launches = 0
    with ClockSampler(local) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        barrier(world)
        ev0.record(stream)
        for _ in range(args.steps):
            st, nc = step()
            launches += st.launches
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = max_over_ranks(ms, world)
    kst = KSTOP.get(args.workload, 0)
    if kst:
        kdone = int(np.sum(nc[:int(np.count_nonzero(nc))]))
        F = flops_k(m, n, kdone) if kdone < min(m, n) else flops_full(m, n)
    else:
        F = flops_full(m, n)
    value = world * F / (ms / 1e3) / 1e12
    clocks = clk.summary()

    out = None
    if rank == 0:
        # instrumented step: per-phase device times (CUDA events on the
        # launching stream) for the roofline of the dominant phase
        sti = Stats()
        sti.timing = 1
        _, nc_i = step(sti)
        peaks, peak_kind = load_peaks()
        phase = {"select": sti.ms_select, "panel": sti.ms_panel, "tfactor": sti.ms_tfactor,
                 "trail": sti.ms_trail, "norm": sti.ms_norm}
        pcy = (C.c_ulonglong * 12)()
        L.qrdm_panel_phase_cycles(pcy, 12)
        if pcy[7]:
            pnames = ["block_sync", "derive_wait", "grid_barrier", "totals", "scalars_wait", "apply",
                      "partials_wait", None, "scalars_own", "derive_own", "partials_own"]
            phase["panel_cta_share"] = {nm: pcy[k] / pcy[7] for k, nm in enumerate(pnames) if nm}
        nblk = int(sti.nblocks)
        if prec == 0:
            # FP64 GEMMs against the best FP64 rate measured on this GPU
            achieved = sti.trail_flops / (sti.ms_trail / 1e3) / 1e12 if sti.ms_trail > 0 else 0.0
            p64, p64_kind = fp64_peak()
            roof = {"bound": "fp64", "kernel": "trailing update (k_trail_w_partial + "
                    "k_trail_w_reduce + k_trail_update), FP64", "achieved": achieved,
                    "peak": p64, "peak_kind": p64_kind,
                    "unit": "TFLOP/s", "frac": achieved / p64,
                    "traffic": load_traffic("trail_fp64"),
                    "per_launch_basis": f"4 m' n' k flops per DM block, {nblk} blocks"}
        else:
            # Ozaki split: s digits per operand, the s (s + 1) / 2 digit
            # products of level <= s + 1 are FP16 GEMMs of the FP64 shape
            # (FP16 and BF16 dense tensor rates are equal on this GPU: the
            # measured BF16 GEMM peak is the denominator).  The update also
            # streams C through HBM (GEMM 1 reads it, GEMM 2 reads and
            # writes it: 24 algorithmic bytes per C entry and block); the
            # bound is whichever roof takes longer for this workload.
            s_dig = int(args.slices or default_options().slices) or 7
            prods = s_dig * (s_dig + 1) // 2
            tflop = sti.trail_flops * prods
            ncv = [int(x) for x in nc_i[:int(np.count_nonzero(nc_i))]]
            entries, jb = 0.0, 0
            for kb in ncv:
                entries += float(m - jb) * float(max(0, n - jb - kb))
                jb += kb
            peak_t = peaks.get("bf16_tflops_sustained")
            peak_b = peaks.get("hbm_gbs")
            t_tensor = tflop / (peak_t * 1e12)
            t_hbm = 24.0 * entries / (peak_b * 1e9)
            sec = sti.ms_trail / 1e3
            tr = load_traffic("trail_ozaki")
            common = {"kernel": "Ozaki trailing update (k_oz_slice_v, k_oz_gemm1, k_oz_vtv + k_larft, "
                                "k_oz_w2, k_oz_gemm2), FP16 tcgen05",
                      "traffic": tr * entries / max(nblk, 1) if tr else None,
                      "traffic_basis": "bytes per DM block (one launch of each kernel): 25.5 B per C "
                                       "entry measured on the first 20 blocks of the 16384 x 8192 "
                                       "workload (profiles/oz_trailing_update_lowrank16k.md) x the "
                                       "average C entries of this workload's blocks",
                      "fp64_equivalent_tflops": sti.trail_flops / sec / 1e12 if sec > 0 else 0.0,
                      "tensor_frac": (tflop / sec / 1e12) / peak_t if sec > 0 else 0.0,
                      "hbm_frac": (24.0 * entries / sec / 1e9) / peak_b if sec > 0 else 0.0}
            if t_tensor >= t_hbm:
                achieved = tflop / sec / 1e12 if sec > 0 else 0.0
                roof = {"bound": "tensor", "achieved": achieved, "peak": peak_t,
                        "peak_kind": f"{peak_kind} bf16 sustained (the phase runs inside a long step)",
                        "unit": "TFLOP/s", "frac": achieved / peak_t,
                        "per_launch_basis": f"{prods} FP16 digit products x 4 m' n' k flops per DM "
                                            f"block, {nblk} blocks"}
            else:
                achieved = 24.0 * entries / sec / 1e9 if sec > 0 else 0.0
                roof = {"bound": "hbm", "achieved": achieved, "peak": peak_b,
                        "peak_kind": f"{peak_kind} HBM copy bandwidth", "unit": "GB/s",
                        "frac": achieved / peak_b,
                        "per_launch_basis": f"24 B per C entry (read by GEMM 1, read and written by "
                                            f"GEMM 2) x m' (n' - k) per DM block, {nblk} blocks"}
            roof.update(common)
        # accuracy of the instrumented factorisation, on the device:
        # ||A P - Q R||_F / ||A||_F with Q R formed by the library's DORMQR,
        # ||I - Q^T Q||_F of the economy Q (the library's DORMQR applied to
        # the first min(m, n) identity columns), and the |R_kk| profile
        accuracy = None
        gpu_jpvt = jp.cpu().numpy().copy()
        gpu_ncols = np.array(nc_i, copy=True)
        gpu_rdiag = torch.abs(torch.diagonal(work.T)[:min(m, n, CPU_SAMPLE_K)]).cpu().numpy()
        try:
            k = int(np.sum(nc_i[:int(np.count_nonzero(nc_i))])) if KSTOP.get(args.workload) else min(m, n)
            k = min(k, m, n)
            Af = work.T  # m x n view of the column-major factor
            R = torch.zeros_like(Af)
            R[:k, :] = torch.triu(Af[:k, :])
            if k < min(m, n):
                R[k:, k:] = Af[k:, k:]
            QR = R.T.contiguous()  # column-major m x n
            del R
            rq = L.qrdm_dormqr_dev(102, m, n, k, C.c_void_p(work.data_ptr()), m, C.c_void_p(tau.data_ptr()),
                                   C.c_void_p(QR.data_ptr()), m)
            if rq == 0:
                p = (jp.long() - 1)
                be = float(torch.linalg.norm(QR - pristine[p]) / torch.linalg.norm(pristine))
                del QR
                mn = min(m, n)
                qt = torch.zeros((mn, m), dtype=torch.float64, device="cuda")  # column-major m x mn
                qt[torch.arange(mn, device="cuda"), torch.arange(mn, device="cuda")] = 1.0
                rq2 = L.qrdm_dormqr_dev(102, m, mn, k, C.c_void_p(work.data_ptr()), m,
                                        C.c_void_p(tau.data_ptr()), C.c_void_p(qt.data_ptr()), m)
                orth = None
                if rq2 == 0:
                    g = qt @ qt.T  # Q^T Q
                    g.diagonal().sub_(1.0)
                    orth = float(torch.linalg.norm(g))
                    del g
                del qt
                rd = torch.abs(torch.diagonal(Af)[:k]).cpu().numpy()
                r0 = float(rd[0]) if rd.size else 0.0
                accuracy = {"backward": be, "backward_bound_10_n_eps": 10 * max(m, n) * 2.0 ** -53,
                            "orth": orth, "orth_bound_100_n_eps": 100 * max(m, n) * 2.0 ** -53,
                            "orth_basis": f"||I - Q^T Q||_F of the economy Q (m x {min(m, n)})",
                            "rkk_first": r0, "rkk_at": {str(i): float(rd[i]) for i in
                                                        (min(k - 1, 2047), min(k - 1, 2048), k - 1)},
                            "numerical_rank_1e-8": int(np.count_nonzero(rd > 1e-8 * r0))}
            else:
                del QR
        except Exception as exc:  # accuracy is reported, never fatal for the timing
            accuracy = {"error": str(exc)[:200]}
        torch.cuda.empty_cache()
        # e2e through the host C ABI with pinned host buffers
        a_host = torch.empty((n, m), dtype=torch.float64, pin_memory=True)
        a_host.copy_(pristine)
        a_np = a_host.numpy()
        src = a_np.copy()
        jp_h = np.zeros(n, np.int32)
        tau_h = np.zeros(min(m, n))
        e2e_t = []
        for it in range(2):
            a_np[...] = src
            jp_h[:] = 0
            nc = np.zeros(n, np.int32)
            opt = default_options(precision=prec, kstop=KSTOP.get(args.workload, 0), slices=args.slices)
            st = Stats()
            t0 = time.perf_counter()
            info = L.dgeqrdm_ex(102, m, n, a_np.ctypes.data_as(pd), m,
                                jp_h.ctypes.data_as(C.POINTER(C.c_int)), tau_h.ctypes.data_as(pd),
                                nc.ctypes.data_as(C.POINTER(C.c_int)), thres.ctypes.data_as(pd),
                                NB, C.byref(opt), C.byref(st))
            e2e_t.append(time.perf_counter() - t0)
            assert info == 0, info
        bytes_io = 8 * m * n + 4 * n + 8 * min(m, n)
        e2e = {"value": world * F / min(e2e_t) / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io}
        variants = {}
        if args.variants:
            if prec != 0:
                st64 = Stats()
                st64.timing = 1
                step(st64, precision=0)
                variants["fp64_dmqr_ms"] = st64.ms_total
                variants["fp64_dmqr_tflops"] = F / (st64.ms_total / 1e3) / 1e12
            if args.workload in SELECTION_BASES:
                # selection property: no base column chosen twice among the first k
                step(precision=prec)
                bid = SELECTION_BASES[args.workload]
                k = KSTOP[args.workload]
                sel = bid[jp[:k].cpu().numpy().astype(np.int64) - 1]
                sel = sel[sel >= 0]
                variants["selected_bases"] = int(len(sel))
                variants["distinct_bases"] = bool(len(np.unique(sel)) == len(sel))
        if args.variants and args.workload not in KSTOP:
            # GPU QP3 (dgeqp3 semantics) on the same matrix, one run
            work.copy_(pristine)
            jp.zero_()
            q0 = torch.cuda.Event(enable_timing=True)
            q1 = torch.cuda.Event(enable_timing=True)
            q0.record(stream)
            rq = L.dgeqp3_dev(102, m, n, C.c_void_p(work.data_ptr()), m,
                              C.c_void_p(jp.data_ptr()), C.c_void_p(tau.data_ptr()))
            q1.record(stream)
            torch.cuda.synchronize()
            if rq == 0:
                variants["qp3_ms"] = q0.elapsed_time(q1)
                variants["qp3_tflops"] = F / (variants["qp3_ms"] / 1e3) / 1e12
                variants["speedup_vs_qp3"] = variants["qp3_ms"] / ms
        if args.variants:
            if "fp64_dmqr_ms" in variants:
                variants["speedup_vs_fp64"] = variants["fp64_dmqr_ms"] / ms
            variants["phase_ms"] = phase
            variants["blocks"] = nblk
            variants["fp64_rates_tflops"] = fp64_rates()
            variants["legacy_mma_rates"] = legacy_mma_rates()
            if args.workload == "lowrank16k" and args.configs:
                variants["configs"] = other_configs(L, stream)
        cpu = None
        if args.cpu_baseline:
            threads = os.cpu_count() or 1
            s = cpu_sample(args.workload, threads, pristine.cpu().numpy(), margins=True)
            cpu = {"value": s["value"], "unit": "TFLOP/s", "cores": threads, "kind": "port",
                   "sample": f"{args.workload} factored until >= {CPU_SAMPLE_K} columns "
                             f"(k={s['k']}, {s['seconds']:.1f} s), oracle port of the reference "
                             "on OpenBLAS, all host threads"}
            # the same oracle run pins the GPU factorisation's choices
            try:
                par = parity_vs_oracle(s["run"], gpu_jpvt, gpu_ncols, gpu_rdiag)
            except Exception as exc:
                par = {"error": str(exc)[:200]}
            if accuracy is None or "error" in accuracy:
                accuracy = {"error": (accuracy or {}).get("error")}
            accuracy["parity"] = par
        out = {"metric": "DM-QR effective FP64 TFLOP/s", "value": value, "unit": "TFLOP/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic",
               "config": {"workload": args.workload, "m": m, "n": n, "nb": NB, "delta": DELTA,
                          "tau_": TAU_, "precision": args.precision, "matrix": desc,
                          "kstop": KSTOP.get(args.workload, 0), "slices": args.slices or None,
                          "parallelism": f"replicas{world}",
                          "l2": "inputs (8 m n bytes) larger than L2; no flush needed"},
               "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
               "gpu_launches": launches, "clocks": clocks, "accuracy": accuracy, "variants": variants}
        print(json.dumps(out), flush=True)
    barrier(world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return out


# ------------------------------------------------------------------ batched
def batched_problem_device(i, m, n, seed=4):
    """Matrix i of the batched workload on the GPU (torch, seeded): U (m x n)
    and V (n x n) orthonormal from Gaussians, s geometric from 1 to 10^-d,
    d ~ U[4, 14].  Returned column-major as a flat float64 tensor."""
    import torch

    g = torch.Generator(device="cuda").manual_seed(seed * 1000003 + i)
    d = 4.0 + 10.0 * torch.rand(1, generator=g, dtype=torch.float64, device="cuda")
    u, _ = torch.linalg.qr(torch.randn(m, n, generator=g, dtype=torch.float64, device="cuda"))
    v, _ = torch.linalg.qr(torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda"))
    k = torch.arange(n, dtype=torch.float64, device="cuda")
    s = torch.pow(10.0, -d * k / max(n - 1, 1))
    a = (u * s) @ v.T
    return a.T.contiguous().view(-1)


def batched_setup(seed=4, count=None):
    import torch

    from qrdm_gb300 import BatchedDMQR
    from qrdm_gb300.workloads import batched_shapes

    ms, ns = batched_shapes(count or BATCH_COUNT, seed=seed)
    shapes = [(int(m), int(n)) for m, n in zip(ms, ns)]
    b = BatchedDMQR(shapes)
    global BATCH_GENERATOR
    try:
        for i, (m, n) in enumerate(shapes):
            b.a[b.a_off[i]:b.a_off[i + 1]] = batched_problem_device(i, m, n, seed)
        BATCH_GENERATOR = "torch (GPU QR of seeded Gaussians)"
    except RuntimeError:
        # torch's GPU linear algebra can be unavailable (e.g. under a
        # profiler): same distribution from the host generator
        from qrdm_gb300.workloads import batched_matrix

        b.load([batched_matrix(i, m, n, seed) for i, (m, n) in enumerate(shapes)])
        BATCH_GENERATOR = "numpy (host QR of seeded Gaussians)"
    torch.cuda.synchronize()
    return b, shapes


OZ_PRODUCTS_BATCHED = 28  # digit products per FP64 MAC in the batched kernel (7 digits, levels <= 8)


def batched_roofline(shapes, ncols_all, v_off, mixed, p64, ptc, bw):
    """Summed per-problem roofline of the batched launch, on the arithmetic
    each phase actually uses, from the DM block sizes the run produced
    (problem i's blocks k_1, k_2, ... at column j with m' = m - j, n' = n - j):
      FP64 pipe: the panel 2 m' k^2 - 2 k^3 / 3, the T recurrence k^3 / 3,
        W2 = T^T W k^2 (n' - k), the norm downdate 2 k (n' - k); in the FP64
        form also the products below;
      tensor pipe (mixed form): the trailing update 4 m' (n' - k) k and V^T V
        m' k^2, each as 28 FP16 digit products, and the BF16 cosine Gram
        2 m' k^2 (k candidates at least);
      HBM: 16 m n bytes (the matrix read and written once).
    Problem time = max(FP64 / P64, tensor / Ptc, bytes / BW); returns
    (sum of problem times in s, FP64 flops, tensor flops)."""
    t = f64_all = ftc_all = 0.0
    for i, (m, n) in enumerate(shapes):
        blocks = np.asarray(ncols_all[int(v_off[i]):int(v_off[i + 1])], dtype=np.float64)
        blocks = blocks[blocks > 0]
        a64 = atc = 0.0
        j = 0.0
        for kb in blocks:
            mp, nn = m - j, n - j
            rest = max(0.0, nn - kb)
            a64 += 2.0 * mp * kb * kb - 2.0 * kb ** 3 / 3.0 + kb ** 3 / 3.0 + kb * kb * rest + 2.0 * kb * rest
            prod = 4.0 * mp * rest * kb + mp * kb * kb
            gram = 2.0 * mp * kb * kb
            if mixed:
                atc += OZ_PRODUCTS_BATCHED * prod + gram
            else:
                a64 += prod + gram
            j += kb
        t += max(a64 / (p64 * 1e12), atc / (ptc * 1e12), 16.0 * m * n / (bw * 1e9))
        f64_all += a64
        ftc_all += atc
    return t, f64_all, ftc_all


def batched_errors(b, pristine):
    """Per-problem backward error ||A P - Q R||_F / ||A||_F and orthogonality
    ||I - Q^T Q||_F on the GPU (torch Householder product of the factors)."""
    import torch

    a_out = b.a
    jp = b.jpvt.cpu().numpy()
    be, orth = [], []
    for i, (m, n) in enumerate(b.shapes):
        k = min(m, n)
        A0 = pristine[b.a_off[i]:b.a_off[i + 1]].view(n, m).T
        F = a_out[b.a_off[i]:b.a_off[i + 1]].view(n, m).T
        tau = b.tau[b.t_off[i]:b.t_off[i] + k]
        Q = torch.linalg.householder_product(F[:, :k], tau)
        R = torch.triu(F[:k, :])
        perm = torch.from_numpy(jp[b.v_off[i]:b.v_off[i + 1]].astype(np.int64) - 1).cuda()
        AP = A0[:, perm]
        be.append(float(torch.linalg.norm(AP - Q @ R) / torch.linalg.norm(A0)))
        orth.append(float(torch.linalg.norm(torch.eye(k, dtype=torch.float64, device="cuda") - Q.T @ Q)))
    return np.array(be), np.array(orth)


def batched_cpu_sample(b_shapes, pristine_host, offs, threads, seed=7, nb=BATCH_NB):
    """Oracle DM-QR over a seeded random sample of the batch's problems."""
    from oracle.oracle import Oracle, run_dmqr

    rng = np.random.default_rng(seed)
    idx = rng.choice(len(b_shapes), size=min(BATCH_CPU_SAMPLE, len(b_shapes)), replace=False)
    o = Oracle(threads=threads)
    mats = []
    for i in idx:
        m, n = b_shapes[i]
        mats.append(pristine_host[offs[i]:offs[i + 1]].reshape(n, m).T)
    t0 = time.perf_counter()
    for A0 in mats:
        r = run_dmqr(o, A0, nb=nb, delta=DELTA, tau_=TAU_)
        assert r["info"] == 0
    dt = time.perf_counter() - t0
    return {"value": len(mats) / dt, "seconds": dt, "problems": len(mats)}


def batched_measure(L, stream, steps, warmup, count=None, batch_nb=0, precision="mixed",
                    cpu_baseline=False, world=1, clocks=False, local=0):
    """The batched workload: one step = one persistent launch factoring the
    whole batch (device-resident, restored from a pristine copy inside the
    timed region).  Returns the measurement dict (rank-local timing)."""
    import torch

    b, shapes = batched_setup(count=count)
    n_prob = len(shapes)
    pristine = b.a.clone()
    tuned = None
    if batch_nb > 0:
        bnb, bprec = batch_nb, precision
    else:
        # block size and arithmetic from the autotuner (timed on a sample of
        # the batch's shapes)
        from qrdm_gb300.autotune import tune_batched

        tuned = tune_batched(shapes, delta=DELTA, tau_=TAU_)
        bnb, bprec = tuned["nb"], tuned["precision"]

    def step():
        b.a.copy_(pristine)
        r = b.run(nb=bnb, delta=DELTA, tau_=TAU_, precision=bprec)
        if r != 0:
            raise RuntimeError(f"dgeqrdm_batched_dev returned {r}")

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    clk = ClockSampler(local) if clocks else None
    if clk:
        clk.__enter__()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier(world)
    ev0.record(stream)
    for _ in range(steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    if clk:
        clk.__exit__()
    ms = max_over_ranks(ev0.elapsed_time(ev1) / steps, world)
    out = {"ms": ms, "count": n_prob, "nb": bnb, "precision": bprec, "autotune": tuned,
           "value": world * n_prob / (ms / 1e3), "clocks": clk.summary() if clk else None}
    peaks, peak_kind = load_peaks()
    F = sum(flops_full(m, n) for m, n in shapes)
    # kernel-only time of the persistent launch (events around the run)
    b.a.copy_(pristine)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.run(nb=bnb, delta=DELTA, tau_=TAU_, precision=bprec)
    e1.record(stream)
    torch.cuda.synchronize()
    kms = e0.elapsed_time(e1)
    cyc = (C.c_ulonglong * 9)()
    L.qrdm_batched_phase_cycles(cyc, 9)
    names = ["norms", "select", "panel", "tfactor", "trail", "downdate", "queue"]
    busy = float(cyc[7]) or 1.0
    phases = {nm: float(cyc[k]) / busy for k, nm in enumerate(names)}
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    phases["longest_over_mean_cta"] = float(cyc[8]) / (busy / nsm)
    p64, p64_kind = fp64_peak()
    ptc = peaks.get("bf16_tflops")
    nc_all = b.ncols.cpu().numpy()
    t_roof, f64, ftc = batched_roofline(shapes, nc_all, b.v_off, bprec == "mixed", p64, ptc,
                                        peaks["hbm_gbs"])
    try:
        be, orth = batched_errors(b, pristine)
    except RuntimeError:  # torch's GPU linear algebra unavailable
        be, orth = np.full(1, np.nan), np.full(1, np.nan)
    out["roofline"] = {
        "bound": "summed per-problem roof (FP64 pipe, tensor pipe, HBM)",
        "kernel": "k_dmqr_batched (one persistent launch; trailing update, V^T V and Gram on " +
                  ("FP16/BF16 tensor cores" if bprec == "mixed" else "the FP64 pipe") + ")",
        "achieved": n_prob / (kms / 1e3), "peak": n_prob / t_roof, "unit": "matrices/s",
        "frac": t_roof / (kms / 1e3),
        "peaks": {"fp64_tflops": p64, "fp64_kind": p64_kind, "tensor_tflops": ptc,
                  "tensor_kind": f"{peak_kind} bf16 burst (FP16 rate equal)",
                  "hbm_gbs": peaks["hbm_gbs"]},
        "fp64_flops": f64, "tensor_flops": ftc, "fp64_equivalent_flops": F,
        "effective_fp64_tflops": F / (kms / 1e3) / 1e12,
        "traffic": load_traffic("dmqr_batched"),
        "per_launch_basis": f"{n_prob} problems; per problem max(FP64 work / P64, tensor work / "
                            "Ptc, 16 m n B / BW) over its actual DM blocks"}
    out["kernel_ms"] = kms
    out["phase_share"] = phases
    out["errors"] = {"backward_p50": float(np.percentile(be, 50)),
                     "backward_p99": float(np.percentile(be, 99)),
                     "backward_max": float(be.max()),
                     "orth_p50": float(np.percentile(orth, 50)),
                     "orth_p99": float(np.percentile(orth, 99))}
    # e2e: pinned host buffer -> device, factor, factors back to the host
    host = torch.empty(pristine.numel(), dtype=torch.float64, pin_memory=True)
    host.copy_(pristine)
    back = torch.empty_like(host)
    e2e_t, parts = [], []
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for _ in range(4):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev[0].record()
        b.a.copy_(host, non_blocking=True)
        ev[1].record()
        b.run(nb=bnb, delta=DELTA, tau_=TAU_, precision=bprec)
        ev[2].record()
        back.copy_(b.a, non_blocking=True)
        ev[3].record()
        b.jpvt.cpu()
        b.tau.cpu()
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
        parts.append([ev[q].elapsed_time(ev[q + 1]) for q in range(3)])
    h2d = 8 * pristine.numel()
    d2h = 8 * pristine.numel() + 4 * b.jpvt.numel() + 8 * b.tau.numel()
    best = int(np.argmin(e2e_t))
    out["e2e"] = {"value": world * n_prob / e2e_t[best], "unit": "matrices/s",
                  "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                  "ms_h2d_factor_d2h": [round(x, 2) for x in parts[best]],
                  "ms_all": [round(1e3 * x, 1) for x in e2e_t]}
    out["flops"] = F
    out["bytes"] = 8 * pristine.numel()
    out["cpu"] = None
    if cpu_baseline:
        threads = os.cpu_count() or 1
        sc = batched_cpu_sample(shapes, pristine.cpu().numpy(), b.a_off, threads, nb=bnb)
        out["cpu"] = {"value": sc["value"], "unit": "matrices/s", "cores": threads, "kind": "port",
                      "sample": f"{sc['problems']} problems of the batch drawn by seed, factored one "
                                f"after another by the oracle port on OpenBLAS ({sc['seconds']:.1f} s)"}
    del b, pristine, host, back
    torch.cuda.empty_cache()
    return out


def run_batched(args):
    import torch

    from qrdm_gb300 import lib

    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    L = lib()
    stream = torch.cuda.current_stream()
    L.qrdm_set_stream(C.c_void_p(stream.cuda_stream))
    r = batched_measure(L, stream, args.steps, args.warmup, count=args.count, batch_nb=args.batch_nb,
                        precision=args.precision, cpu_baseline=args.cpu_baseline and rank == 0,
                        world=world, clocks=True, local=local)
    if rank == 0:
        out = {"metric": "batched DM-QR matrices/s", "value": r["value"], "unit": "matrices/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"],
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic",
               "config": {"workload": "batched2000", "count": r["count"], "nb": r["nb"],
                          "precision": r["precision"], "autotune": r["autotune"],
                          "delta": DELTA, "tau_": TAU_, "flops": r["flops"], "generator": BATCH_GENERATOR,
                          "bytes": r["bytes"], "parallelism": f"replicas{world}",
                          "l2": "inputs (3.3 GB) larger than L2; no flush needed"},
               "roofline": r["roofline"], "cpu_baseline": r["cpu"], "e2e": r["e2e"],
               "gpu_launches": args.steps, "clocks": r["clocks"],
               "phase_share": r["phase_share"], "errors": {**r["errors"], "kernel_ms": r["kernel_ms"]}}
        print(json.dumps(out), flush=True)
    barrier(world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_batched_reference(args):
    import torch

    rank, world, _ = dist_setup(args.gpus)
    if rank != 0:
        return
    b, shapes = batched_setup()
    host = b.a.cpu().numpy()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        batched_cpu_sample(shapes, host, b.a_off, threads)
    vals, secs = [], []
    for _ in range(args.steps):
        s = batched_cpu_sample(shapes, host, b.a_off, threads)
        vals.append(s["value"])
        secs.append(s["seconds"])
    v = statistics.median(vals)
    sample = (f"{s['problems']} problems of the 2000-matrix batch drawn by seed, oracle port of "
              "the reference on OpenBLAS, one after another")
    print(json.dumps({
        "impl": "reference", "metric": "batched DM-QR matrices/s", "value": v,
        "unit": "matrices/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.median(secs) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "batched2000", "count": BATCH_COUNT, "nb": BATCH_NB},
        "cpu_baseline": {"value": v, "unit": "matrices/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "matrices/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="lowrank16k")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--no-variants", dest="variants", action="store_false")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="default workload: skip the one-step measurements of the other configurations")
    ap.add_argument("--count", type=int, default=None,
                    help="batched2000: number of problems (default 2000)")
    ap.add_argument("--slices", type=int, default=0,
                    help="mixed precision: digits per operand of the Ozaki split (0: library default)")
    ap.add_argument("--batch-nb", type=int, default=0,
                    help="batched2000: DM block size (0: autotuner picks nb and precision)")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-full-run", dest="full_run", action="store_false",
                    help="reference arm: skip the one whole factorisation beside the timed samples")
    args = ap.parse_args()
    if args.workload == "batched2000":
        if args.impl == "reference":
            run_batched_reference(args)
        else:
            run_batched(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
