"""Benchmark of the GB300 DM-QR hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload lowrank16k|gauss4k|kahan4k|graded1k]
                    [--precision mixed|fp64] [--no-variants]

One step = one DM-QR factorisation of the workload matrix, already resident
in HBM (restored from a pristine device copy before each step; the copy is
inside the timed region).  The default workload is the 16384 x 8192
numerical-rank-2048 matrix A = L R^T + 1e-10 E (full factorisation, nb = 64,
delta = 0.9, tau_ = 0.15).  Inputs (1.07 GB) are larger than the 129 MB L2,
so no explicit flush is needed between steps.

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
}
NB, DELTA, TAU_ = 64, 0.9, 0.15
CPU_SAMPLE_K = 2048


def flops_full(m, n):
    return 2.0 * m * n * n - 2.0 * n ** 3 / 3.0 if m >= n else 2.0 * n * m * m - 2.0 * m ** 3 / 3.0


def flops_k(m, n, k):
    return 4.0 * m * n * k - 2.0 * (m + n) * k * k + 4.0 * k ** 3 / 3.0


def make_matrix_device(name, seed=3):
    """Column-major workload matrix as a CUDA float64 tensor of shape (n, m)."""
    import torch

    m, n, _ = WORKLOADS[name]
    g = torch.Generator(device="cuda").manual_seed(seed)
    dev = "cuda"
    if name == "lowrank16k":
        r = 2048
        lf = torch.randn(m, r, generator=g, dtype=torch.float64, device=dev) / math.sqrt(r)
        rf = torch.randn(n, r, generator=g, dtype=torch.float64, device=dev) / math.sqrt(r)
        at = rf @ lf.T
        at += 1e-10 * torch.randn(n, m, generator=g, dtype=torch.float64, device=dev)
        return at.contiguous()
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

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
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

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


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


def cpu_sample(name, threads, at_host=None):
    """Oracle (CPU restatement of the reference, OpenBLAS) on the bounded
    sample: the workload matrix factored until >= CPU_SAMPLE_K columns."""
    from oracle.oracle import Oracle, run_dmqr

    m, n, _ = WORKLOADS[name]
    if at_host is None:
        at_host = make_matrix_device(name).cpu().numpy()
    A0 = at_host.T  # Fortran-ordered m x n view
    o = Oracle(threads=threads)
    k_target = min(CPU_SAMPLE_K, min(m, n))
    t0 = time.perf_counter()
    r = run_dmqr(o, A0, nb=NB, delta=DELTA, tau_=TAU_, kstop=k_target)
    dt = time.perf_counter() - t0
    k = int(np.sum(r["ncols"]))
    f = flops_k(m, n, k) if k < min(m, n) else flops_full(m, n)
    return {"value": f / dt / 1e12, "seconds": dt, "k": k, "flops": f}


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
    line = {"impl": "reference", "metric": "DM-QR effective FP64 TFLOP/s", "value": v,
            "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.median(secs) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "m": m, "n": n, "nb": NB, "delta": DELTA,
                       "tau_": TAU_, "matrix": desc, "sample_columns": s["k"]},
            "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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
        opt = default_options(precision=precision)
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
    F = flops_full(m, n)
    value = world * F / (ms / 1e3) / 1e12
    clocks = clk.summary()

    out = None
    if rank == 0:
        # instrumented step: per-phase device times (CUDA events on the
        # launching stream) for the roofline of the dominant phase
        sti = Stats()
        sti.timing = 1
        step(sti)
        peaks, peak_kind = load_peaks()
        phase = {"select": sti.ms_select, "panel": sti.ms_panel, "tfactor": sti.ms_tfactor,
                 "trail": sti.ms_trail, "norm": sti.ms_norm}
        nblk = int(sti.nblocks)
        if prec == 0:
            # FP64 FMA GEMMs: no measured FP64 peak exists for this machine;
            # GB300's nominal dense FP64 rate is used
            achieved = sti.trail_flops / (sti.ms_trail / 1e3) / 1e12
            roof = {"bound": "tensor", "kernel": "trailing update (k_trail_w_partial + "
                    "k_trail_w_reduce + k_trail_update), FP64 FMA", "achieved": achieved,
                    "peak": 1.25, "peak_kind": "nominal FP64 (no measured FP64 peak)",
                    "unit": "TFLOP/s", "frac": achieved / 1.25,
                    "traffic": load_traffic("trail_fp64"),
                    "per_launch_basis": f"4 m' n' k flops per DM block, {nblk} blocks"}
        else:
            achieved = sti.trail_flops / (sti.ms_trail / 1e3) / 1e12
            roof = {"bound": "tensor", "kernel": "Ozaki trailing update", "achieved": achieved,
                    "peak": peaks.get("bf16_tflops"), "peak_kind": peak_kind,
                    "unit": "TFLOP/s", "frac": None, "traffic": load_traffic("trail_ozaki")}
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
            opt = default_options(precision=prec)
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
                st64, _ = step(precision=0)
                variants["fp64_dmqr_ms"] = st64.ms_total
                variants["fp64_dmqr_tflops"] = F / (st64.ms_total / 1e3) / 1e12
            variants["phase_ms"] = phase
            variants["blocks"] = nblk
        cpu = None
        if args.cpu_baseline:
            threads = os.cpu_count() or 1
            s = cpu_sample(args.workload, threads, pristine.cpu().numpy())
            cpu = {"value": s["value"], "unit": "TFLOP/s", "cores": threads, "kind": "port",
                   "sample": f"{args.workload} factored until >= {CPU_SAMPLE_K} columns "
                             f"(k={s['k']}, {s['seconds']:.1f} s), oracle port of the reference "
                             "on OpenBLAS, all host threads"}
        out = {"metric": "DM-QR effective FP64 TFLOP/s", "value": value, "unit": "TFLOP/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic",
               "config": {"workload": args.workload, "m": m, "n": n, "nb": NB, "delta": DELTA,
                          "tau_": TAU_, "precision": args.precision, "matrix": desc,
                          "parallelism": f"replicas{world}",
                          "l2": "inputs (8 m n bytes) larger than L2; no flush needed"},
               "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
               "gpu_launches": launches, "clocks": clocks, "variants": variants}
        print(json.dumps(out), flush=True)
    barrier(world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="lowrank16k")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="fp64")
    ap.add_argument("--no-variants", dest="variants", action="store_false")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
