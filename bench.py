"""Benchmark: two-site H*psi matvec at bond dimension D=4000 (U(1) spin-1/2 chain,
Sz sectors -30..30 with Gaussian dims sigma=9, physical d=2, MPO bond w=5), seconds per
matvec, in the plain FP64 form and the split-precision form.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--mode split|fp64]

One step = one application of H_eff to psi, i.e. the reference's four-Contract chain
(tests/test_tensor_manipulation/test_ten_ctrct_1sct.cc:253-257). Inputs are synthetic
tensors with the reference case's shapes (seeded N(0,1), psi normalised), generated by
tensortoolkit_gb300/csrc/synth.h; no dataset is involved.

value  : device-resident time per matvec (graph launch only), L2 flushed between steps.
e2e    : the same through the public API with host buffers - pinned host psi copied in,
         H_eff psi computed, result copied back - every step.
roofline: the dominant kernel (grouped GEMM) timed with CUDA events on its own stream.
cpu_baseline: the CPU restatement of the reference's algorithm (OpenBLAS dgemm per block
         pair, as the reference's CPU build) on a bounded sample of the same workload.
--impl reference: that CPU path alone, timed over the same steps.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(D=4000, qmax=30, sigma=9.0, seed=1)
WORKLOAD_NAME = "two-site H*psi matvec, U(1) Heisenberg chain, D=4000 (Sz -30..30, sigma 9), d=2, w=5"
METRIC = "two-site H*psi matvec s/iter at D=4000"
L2_FLUSH_BYTES = 512 << 20


def peaks():
    p = {}
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        p["source"] = "measured"
    else:
        p = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}
    return p


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_matvec_time(tensors, iters: int, threads: int) -> float:
    """Seconds per matvec of the CPU restatement (median of `iters`)."""
    from oracle import oracle
    oracle.set_threads(threads)
    lenv, psi, mpo1, mpo2, renv = tensors
    oracle.matvec(lenv, psi, mpo1, mpo2, renv)  # warm-up
    ts = []
    for _ in range(iters):
        t0 = time.perf_counter()
        oracle.matvec(lenv, psi, mpo1, mpo2, renv)
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from tensortoolkit_gb300 import workloads
    tensors = workloads.heisenberg(WORKLOAD["D"], WORKLOAD["qmax"], WORKLOAD["sigma"], WORKLOAD["seed"])
    threads = os.cpu_count() or 1
    from oracle import oracle
    oracle.set_threads(threads)
    for _ in range(args.warmup):
        oracle.matvec(*tensors)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.matvec(*tensors)
        ts.append(time.perf_counter() - t0)
    v = sum(ts) / len(ts)
    out = {"metric": METRIC, "value": v, "unit": "s/iter", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded N(0,1), reference shapes)",
           "config": {"workload": WORKLOAD_NAME, **WORKLOAD}, "impl": "reference",
           "cpu_baseline": {"value": v, "unit": "s/iter", "cores": threads, "kind": "port",
                            "sample": f"{args.steps} full matvecs after {args.warmup} warm-up"},
           "e2e": {"value": v, "unit": "s/iter", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["split", "fp64"], default=os.environ.get("QLTG_BENCH_MODE", "fp64"))
    ap.add_argument("--cpu-iters", type=int, default=None, help="CPU baseline sample size")
    ap.add_argument("--profile", action="store_true",
                    help="profiling run: plan the D=4000 matvec, apply it twice, print nothing else")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch
    import torch.distributed as dist
    from tensortoolkit_gb300 import workloads
    from tensortoolkit_gb300.api import ContractionPlan, DTensor, Matvec, context
    from tensortoolkit_gb300 import capi
    import ctypes as C

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    tensors = workloads.heisenberg(WORKLOAD["D"], WORKLOAD["qmax"], WORKLOAD["sigma"], WORKLOAD["seed"])
    lenv, psi, mpo1, mpo2, renv = tensors
    dl, dp, d1, d2, dr = (DTensor.from_host(x, local) for x in tensors)
    mv = Matvec(dl, psi, d1, d2, dr, mode=args.mode)
    flops, launches_per_step = mv.stats()
    out = DTensor.empty(mv.result, local)
    if args.profile:
        for _ in range(2):
            mv.apply(dp, out)
        torch.cuda.synchronize()
        print(json.dumps({"profile_run": True, "mode": args.mode, "launches_per_step": launches_per_step}))
        return
    stream = torch.cuda.current_stream(local)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")

    # warm-up
    for _ in range(args.warmup):
        mv.apply(dp, out)
    torch.cuda.synchronize()

    # device-resident timed region
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            flush.fill_(float(i))            # write > L2 between steps
            evs[i][0].record(stream)
            mv.apply(dp, out)
            evs[i][1].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    dev_ms = sum(a.elapsed_time(b) for a, b in evs)
    t_step = dev_ms / 1e3 / args.steps

    # end to end through the public API with pinned host buffers
    h_in = torch.from_numpy(psi.raw_f64()).pin_memory()
    h_out = torch.empty(mv.result.size * (2 if mv.result.is_complex else 1), dtype=torch.float64).pin_memory()
    d_in = DTensor.empty(psi, local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(2):
        d_in.buf[: h_in.numel()].copy_(h_in, non_blocking=True)
        mv.apply(d_in, out)
        h_out.copy_(out.buf[: h_out.numel()], non_blocking=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for i in range(args.steps):
        d_in.buf[: h_in.numel()].copy_(h_in, non_blocking=True)
        mv.apply(d_in, out)
        h_out.copy_(out.buf[: h_out.numel()], non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_step = e0.elapsed_time(e1) / 1e3 / args.steps

    # roofline of the dominant kernel: the grouped GEMM of each step, timed alone
    pk = peaks()
    gemm_stats = []
    plans = []
    ins = [dl, None, None, None]
    cur_a = dl
    bs = [dp, d1, d2, dr]
    axes = [[[0], [0]], [[0, 2], [0, 1]], [[4, 1], [0, 1]], [[4, 1], [1, 0]]]
    a_meta = lenv
    outs = []
    for i in range(4):
        p = ContractionPlan(a_meta, bs[i].meta if i else psi, axes[i], local)
        c = DTensor.empty(p.result, local)
        p.execute(cur_a, bs[i], c, mode=args.mode)
        plans.append((p, cur_a, bs[i], c))
        cur_a, a_meta = c, p.result
    torch.cuda.synchronize()
    mode_i = capi.QLTG_MODE_SPLIT if args.mode == "split" else capi.QLTG_MODE_FP64
    gemm_ms_total, gemm_flops_total = 0.0, 0.0
    reps = 5
    for p, a, b, c in plans:
        sp = C.c_void_p(stream.cuda_stream)
        capi.check(capi.lib().qltg_ctrct_exec_stage(p.h, C.c_void_p(a.ptr), C.c_void_p(b.ptr), C.c_void_p(c.ptr),
                                                    mode_i, 1, sp))
        ts = []
        for r in range(reps):
            flush.fill_(float(r))
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            capi.check(capi.lib().qltg_ctrct_exec_stage(p.h, C.c_void_p(a.ptr), C.c_void_p(b.ptr),
                                                        C.c_void_p(c.ptr), mode_i, 2, sp))
            s1.record(stream)
            ts.append((s0, s1))
        torch.cuda.synchronize()
        ms = statistics.median(x.elapsed_time(y) for x, y in ts)
        f, _ = p.stats()
        gemm_stats.append({"flops": f, "ms": ms})
        gemm_ms_total += ms
        gemm_flops_total += f
    # FP64 peak: cuBLAS DGEMM through torch (the plain-FP64 denominator); tensor peak for split
    if args.mode == "fp64":
        n = 8192
        x = torch.randn(n, n, dtype=torch.float64, device=f"cuda:{local}")
        y = torch.randn(n, n, dtype=torch.float64, device=f"cuda:{local}")
        torch.matmul(x, y)
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(3):
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            torch.matmul(x, y)
            s1.record(stream)
            torch.cuda.synchronize()
            best = min(best, s0.elapsed_time(s1))
        peak_tf = 2 * n ** 3 / (best / 1e3) / 1e12
        peak_src = "cuBLAS DGEMM 8192^3 measured in this run (FP64 pipe)"
        del x, y
    else:
        peak_tf = pk["bf16_tflops"]
        peak_src = f"bf16 dense, {pk['source']} (MEASURED_PEAKS.json)"
    achieved = gemm_flops_total / (gemm_ms_total / 1e3) / 1e12
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peak_tf, "unit": "TFLOP/s",
                "frac": achieved / peak_tf if peak_tf else None, "traffic": None,
                "kernel": "k_gemm_grouped (4 launches per matvec)", "peak_source": peak_src,
                "per_step_ms": [round(g["ms"], 4) for g in gemm_stats],
                "gemm_share_of_step": gemm_ms_total / (t_step * 1e3)}

    # max over ranks
    t_max = t_step
    if world > 1:
        tt = torch.tensor([t_step], device=f"cuda:{local}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())

    if rank == 0:
        cpu = None
        cpu_iters = args.cpu_iters
        try:
            if cpu_iters is None:
                cpu_iters = 10
            threads = os.cpu_count() or 1
            v = cpu_matvec_time(tensors, cpu_iters, threads)
            cpu = {"value": v, "unit": "s/iter", "cores": threads, "kind": "port",
                   "sample": f"median of {cpu_iters} full D=4000 matvecs (OpenBLAS dgemm per block pair)"}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "s/iter", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"unavailable: {e}"}
        res = {
            "metric": METRIC, "value": t_max / world, "unit": "s/iter", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "precision": "split (BF16-slice emulated FP64)" if args.mode == "split" else "plain FP64",
            "data": "synthetic (seeded N(0,1) operands with the reference case's shapes)",
            "config": {"workload": WORKLOAD_NAME, **WORKLOAD, "mode": args.mode,
                       "l2": "512 MiB buffer written between timed steps",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "gflops_fp64_equiv": flops / t_step / 1e9,
            "algorithmic_gflop_per_step": flops / 1e9,
            "e2e": {"value": e2e_step, "unit": "s/iter", "h2d_bytes_per_step": int(h_in.numel() * 8),
                    "d2h_bytes_per_step": int(h_out.numel() * 8)},
            "gpu_launches": int(launches_per_step * args.steps),
            "gpu_launches_per_step": int(launches_per_step),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(res))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
