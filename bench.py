"""Benchmark: two-site H*psi matvec at bond dimension D=4000 (U(1) spin-1/2 chain,
Sz sectors -30..30 with Gaussian dims sigma=9, physical d=2, MPO bond w=5), seconds per
matvec, in the plain FP64 form and the split-precision form.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--mode split|fp64]

One step = one application of H_eff to psi, i.e. the reference's four-Contract chain
(tests/test_tensor_manipulation/test_ten_ctrct_1sct.cc:253-257). Inputs are synthetic
tensors with the reference case's shapes (seeded N(0,1), psi normalised), generated by
tensortoolkit_gb300/csrc/synth.h; no dataset is involved.

value  : device-resident time per matvec (graph launch only), L2 flushed between steps.
e2e    : the same through the public API with host buffers (qltg_matvec_apply_host) - pinned
         host psi copied in, H_eff psi computed, result copied back - every step.
roofline: the dominant kernel (grouped GEMM) timed with CUDA events on its own stream:
         algorithmic FP64 flops sum(2mkn) / launch time against the FP64-equivalent peak
         (split: the BF16 peak / 28 slice products; FP64: cuBLAS DGEMM measured in the run);
         sum_T_over_t = sum over the four steps of max(F/P, B/BW) / the matvec time.
cpu_baseline: the CPU restatement of the reference's algorithm (OpenBLAS dgemm per block
         pair, as the reference's CPU build) on a bounded sample of the same workload.
--impl reference: that CPU path alone, timed over the same steps.
"""
from __future__ import annotations

import argparse
import json
import math
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


def bench_config(world: int) -> dict:
    """The workload description both arms print (identical dicts, so the two lines compare)."""
    return {"workload": WORKLOAD_NAME, **WORKLOAD,
            "l2": "GPU arm: 512 MiB buffer written between timed steps",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for line in r.stdout.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def replica_time(t_step: float, world: int, device=None) -> float:
    """The job's time per step with one replica per rank: the max over ranks of each rank's
    time (collective on the default process group; device: where the reduced tensor lives -
    the rank's GPU under NCCL, the CPU under gloo)."""
    if world <= 1:
        return t_step
    import torch
    import torch.distributed as dist
    tt = torch.tensor([t_step], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


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


# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu capture of
# `python bench.py --profile --profile-case step0|step3` (split) and `--profile --mode fp64`
# (summaries: profiles/k_gemm_split_d4000.txt, profiles/k_gemm_dfma_d4000.txt). Keyed by
# matvec step.
NCU_TRAFFIC = {
    "split": {0: 117.4e6, 3: 228.9e6},
    "fp64": {0: 84.6e6, 3: 167.7e6},
}


def _time_events(fn, stream, flush, reps=5):
    import torch
    ts = []
    for r in range(reps):
        flush.fill_(float(r))                       # write > L2 before each timed launch
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        fn()
        s1.record(stream)
        ts.append((s0, s1))
    torch.cuda.synchronize()
    return statistics.median(x.elapsed_time(y) for x, y in ts)


_FP64_PEAK = {}


def fp64_peak_tflops(local, stream) -> float:
    """The FP64 pipe's rate on this GPU: cuBLAS DGEMM 8192^3, best of 3, measured once per run."""
    import torch
    if local not in _FP64_PEAK:
        n = 8192
        x = torch.randn(n, n, dtype=torch.float64, device=f"cuda:{local}")
        y = torch.randn(n, n, dtype=torch.float64, device=f"cuda:{local}")
        torch.matmul(x, y)
        torch.cuda.synchronize()
        best_ms = 1e9
        for _ in range(3):
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            torch.matmul(x, y)
            s1.record(stream)
            torch.cuda.synchronize()
            best_ms = min(best_ms, s0.elapsed_time(s1))
        _FP64_PEAK[local] = 2 * n ** 3 / (best_ms / 1e3) / 1e12
    return _FP64_PEAK[local]


def matvec_step_bounds(tensors, local, peak_tflops, hbm_gbs):
    """Per step of the matvec chain (F_s algorithmic flops, B_s = operand + result bytes) and
    the sum over steps of max(F_s / P, B_s / BW) in ms."""
    from tensortoolkit_gb300.api import ContractionPlan
    lenv, psi, mpo1, mpo2, renv = tensors
    axes = [[[0], [0]], [[0, 2], [0, 1]], [[4, 1], [0, 1]], [[4, 1], [1, 0]]]
    a_meta, out = lenv, []
    for i, b in enumerate((psi, mpo1, mpo2, renv)):
        p = ContractionPlan(a_meta, b, axes[i], local)
        f, nbytes = p.stats()
        out.append((f, nbytes))
        a_meta = p.result
        del p
    t = sum(max(f / (peak_tflops * 1e12), nb / (hbm_gbs * 1e9)) for f, nb in out)
    return out, t * 1e3


def gemm_roofline(mode, lenv, psi, d1, d2, dr, dl, dp, local, stream, flush, pk):
    """Per matvec step: the operand transposes, the GEMM stage (incl. operand slicing) and the
    GEMM kernels alone, each timed with CUDA events on the launching stream with L2 flushed
    before every launch;
    the roofline entry is the largest single launch of the dominant kernel."""
    import ctypes as C
    import torch
    from tensortoolkit_gb300 import capi
    from tensortoolkit_gb300.api import ContractionPlan, DTensor
    mode_i = capi.QLTG_MODE_SPLIT if mode == "split" else capi.QLTG_MODE_FP64
    axes = [[[0], [0]], [[0, 2], [0, 1]], [[4, 1], [0, 1]], [[4, 1], [1, 0]]]
    bs = [dp, d1, d2, dr]
    cur_a, a_meta = dl, lenv
    lib = capi.lib()
    sp = C.c_void_p(stream.cuda_stream)
    per, stage_ms, kern_ms, alg_flops, tc_flops = [], 0.0, 0.0, 0.0, 0.0
    best = None
    step_fb = []                       # per step: (algorithmic flops, operand + result bytes)
    for i in range(4):
        b_meta = bs[i].meta if i else psi
        p = ContractionPlan(a_meta, b_meta, axes[i], local)
        eb = 16 if a_meta.is_complex else 8
        step_fb.append((p.stats()[0], (a_meta.size + b_meta.size + p.result.size) * eb))
        c = DTensor.empty(p.result, local)
        p.tune(cur_a, bs[i], c, mode=mode)        # the matvec's own choice, from the tuner's cache
        p.execute(cur_a, bs[i], c, mode=mode)
        args = (p.h, C.c_void_p(cur_a.ptr), C.c_void_p(bs[i].ptr), C.c_void_p(c.ptr), mode_i)
        ms1 = _time_events(lambda: capi.check(lib.qltg_ctrct_exec_stage(*args, 1, sp)), stream, flush)
        ms2 = _time_events(lambda: capi.check(lib.qltg_ctrct_exec_stage(*args, 2, sp)), stream, flush)
        ms3 = _time_events(lambda: capi.check(lib.qltg_ctrct_exec_stage(*args, 3, sp)), stream, flush)
        p.device_status()
        f, _ = p.stats()
        tcf, useful = 0.0, None
        if mode == "split":
            # 28 slice pairs on 128 x 32 x 32 tile stages (padding included), as scheduled
            stages, useful = p.split_stats()
            tcf = stages * 28 * (2 * 128 * 32 * 32)
        sch = p.schedule()
        per.append({"transpose_ms": round(ms1, 4), "stage_ms": round(ms2, 4), "kernel_ms": round(ms3, 4),
                    "gflop": round(f / 1e9, 4),
                    "tensor_gflop": round(tcf / 1e9, 2), "useful_share": None if useful is None else round(useful, 4),
                    "schedule": {"f64_tile_rows": sch["f64_tile_rows"], "split_stack": sch["split_stack"]}})
        stage_ms += ms2
        kern_ms += ms3
        alg_flops += f
        tc_flops += tcf
        work = tcf if mode == "split" else f
        if f > 1e9 and (best is None or ms3 > best[1]):
            best = (i, ms3, work, f)
        cur_a, a_meta = c, p.result
    i, ms, work, f = best
    exec_tflops = exec_frac = None
    if mode == "split":
        # the slice-pipe peak divided by the 28 slice products each FP64 product needs
        bf16 = pk["bf16_tflops"]
        peak = bf16 / 28.0
        src = (f"bf16 dense burst {bf16:.1f} TFLOP/s ({pk['source']}, MEASURED_PEAKS.json) / 28 slice "
               "products = the FP64-equivalent peak of the split form")
        what = (f"k_gemm_split, one launch (matvec step {i}): algorithmic FP64 flops sum(2mkn) / launch time, "
                "against the BF16 peak / 28")
        exec_tflops = work / (ms / 1e3) / 1e12
        exec_frac = exec_tflops / bf16
    else:
        peak = fp64_peak_tflops(local, stream)
        src = "cuBLAS DGEMM 8192^3 measured in this run (the FP64 pipe)"
        what = f"k_gemm_dfma (+ k_gemm_skinny), one launch (matvec step {i}): algorithmic flops sum(2mkn) / launch time"
    achieved = f / (ms / 1e3) / 1e12
    # whole-matvec bound: per step T_s = max(F_s / P, B_s / BW)
    bw = pk["hbm_gbs"] * 1e9
    t_bound = sum(max(fs / (peak * 1e12), bs_ / bw) for fs, bs_ in step_fb)
    out = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
           "frac": achieved / peak if peak else None, "traffic": NCU_TRAFFIC.get(mode, {}).get(i),
           "kernel": what, "peak_source": src, "launch_ms": round(ms, 4),
           "fp64_equiv_tflops": achieved,
           "sum_T_bound_ms": round(t_bound * 1e3, 4),
           "step_bounds": [{"gflop": round(fs / 1e9, 4), "mbytes": round(bs_ / 1e6, 2),
                            "T_flops_ms": round(fs / (peak * 1e12) * 1e3, 4),
                            "T_bytes_ms": round(bs_ / bw * 1e3, 4)} for fs, bs_ in step_fb],
           "per_step": per, "gemm_stage_ms": round(stage_ms, 4), "gemm_kernels_ms": round(kern_ms, 4)}
    if exec_tflops is not None:
        out["executed_tensor_tflops"] = exec_tflops
        out["executed_tensor_frac"] = exec_frac
        out["executed_note"] = "executed BF16 tensor flops (28 slice pairs on 128x32x32 padded tiles) / launch time / BF16 peak"
    return out


def precision_study(local: int, steps: int = 20):
    """The precision configuration on the symmetric (Hermitian) variant of the D=4000 workload:
    relative Frobenius error of the split-precision matvec vs the plain FP64 path (itself
    parity-tested against the oracle), per block and whole, and the drift of the lowest
    Lanczos Ritz value over `steps` iterations (FP64 full reorthogonalisation on the device)
    from the same normalised N(0,1) psi0."""
    import numpy as np
    from tensortoolkit_gb300 import workloads
    from tensortoolkit_gb300.api import DTensor, Lanczos, Matvec
    tensors = workloads.heisenberg(WORKLOAD["D"], WORKLOAD["qmax"], WORKLOAD["sigma"], WORKLOAD["seed"],
                                   hermitian=True)
    lenv, psi, mpo1, mpo2, renv = tensors
    dl, dp, d1, d2, dr = (DTensor.from_host(x, local) for x in tensors)
    out = {}
    for m in ("fp64", "split"):
        mv = Matvec(dl, psi, d1, d2, dr, mode=m)
        y = mv.apply(dp).to_host()
        e = Lanczos(mv, steps).run(dp, steps)
        mv.device_status()
        out[m] = (y, e)
        del mv
    (y64, e64), (ys, es) = out["fp64"], out["split"]
    blk = []
    for b in range(y64.nblk):
        n = np.linalg.norm(y64.block(b))
        if n > 0:
            blk.append(float(np.linalg.norm(ys.block(b) - y64.block(b)) / n))
    drift = np.abs(es - e64)
    return {"workload": WORKLOAD_NAME + ", symmetric lenv/renv (Hermitian H_eff)",
            "matvec_rel_err": float(np.linalg.norm(ys.raw_f64() - y64.raw_f64()) / np.linalg.norm(y64.raw_f64())),
            "max_block_rel_err": max(blk), "median_block_rel_err": float(np.median(blk)), "blocks": len(blk),
            "lanczos_steps": steps, "e0_fp64": float(e64[-1]), "e0_split": float(es[-1]),
            "max_energy_drift": float(drift.max()), "max_rel_energy_drift": float((drift / np.abs(e64)).max()),
            "energy_drift_per_step": [float(x) for x in drift]}


def svd_group_shapes(t, ldims: int):
    """(rows, cols) of the block-diagonal matrices SVD(t, ldims) factors: blocks grouped by
    the quantum-number flux of their left legs (the reference's grouping key)."""
    import numpy as np
    sgn = [1 if l.dir == 0 else -1 for l in t.legs]
    groups = {}
    for b in range(t.nblk):
        c = t.coords[b]
        flux = tuple(np.sum([sgn[l] * t.legs[l].qns[c[l]] for l in range(ldims)], axis=0).tolist())
        g = groups.setdefault(flux, [set(), set()])
        g[0].add(tuple(c[:ldims].tolist()))
        g[1].add(tuple(c[ldims:].tolist()))
    shapes = []
    for rows, cols in groups.values():
        r = sum(int(np.prod([t.legs[l].dims[x[l]] for l in range(ldims)])) for x in rows)
        cc = sum(int(np.prod([t.legs[ldims + l].dims[x[l]] for l in range(t.rank - ldims)])) for x in cols)
        shapes.append((r, cc))
    return shapes


def time_call(fn, reps: int = 5) -> float:
    """Median wall time of fn() in seconds, device synchronised around each call."""
    import torch
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


class ProxyStep:
    """One contraction in the reference GPU build's call pattern (a labelled proxy, not the
    reference itself): BlockSparseDataTensor::CtrctTwoBSDTAndAssignIn
    (qltensor/blk_spar_data_ten/global_operations.h:895-992) transposes every operand block it
    uses once - cutensorPermute per block (framework/hp_numeric/ten_trans.h:245-349), here a
    plain strided copy (torch permute + contiguous) - then issues one cublasDgemm per task on
    the default stream in task order (framework/hp_numeric/blas_level3.h:797-856): beta 0 for
    the task that creates its output block, 1 after, alpha the task's sign. cuBLAS is reached
    through torch (addmm with out=). Bosonic real FP64 tensors only."""

    def __init__(self, a_meta, b_meta, axes, plan):
        sa = [i for i in range(a_meta.rank) if i not in axes[0]]
        sb = [i for i in range(b_meta.rank) if i not in axes[1]]
        self.perm_a, self.perm_b = sa + list(axes[0]), list(axes[1]) + sb
        self.tasks = [tuple(int(x) for x in t) for t in plan.tasks()]
        self.a_pos = {int(x): i for i, x in enumerate(a_meta.blk_idx())}
        self.b_pos = {int(x): i for i, x in enumerate(b_meta.blk_idx())}
        self.c_pos = {int(x): i for i, x in enumerate(plan.result.blk_idx())}
        self.a_meta, self.b_meta, self.c_meta = a_meta, b_meta, plan.result
        self.a_shapes, self.b_shapes = a_meta.block_shapes(), b_meta.block_shapes()
        self.a_used = sorted({self.a_pos[t[0]] for t in self.tasks})
        self.b_used = sorted({self.b_pos[t[1]] for t in self.tasks})

    def run(self, a_buf, b_buf, c_buf):
        import torch
        at, bt = {}, {}
        for i in self.a_used:
            shp = [int(x) for x in self.a_shapes[i]]
            o = int(self.a_meta.offsets[i])
            at[i] = a_buf[o:o + math.prod(shp)].view(shp).permute(self.perm_a).contiguous()
        for i in self.b_used:
            shp = [int(x) for x in self.b_shapes[i]]
            o = int(self.b_meta.offsets[i])
            bt[i] = b_buf[o:o + math.prod(shp)].view(shp).permute(self.perm_b).contiguous()
        for a_idx, b_idx, c_idx, m, k, n, sign, beta in self.tasks:
            A = at[self.a_pos[a_idx]].view(m, k)
            B = bt[self.b_pos[b_idx]].view(k, n)
            o = int(self.c_meta.offsets[self.c_pos[c_idx]])
            Cb = c_buf[o:o + m * n].view(m, n)
            torch.addmm(Cb, A, B, beta=float(beta), alpha=float(sign), out=Cb)


def run_proxy(local: int, stream, flush, reps: int = 5) -> dict:
    """The plain FP64 matvec at D=4000 in the reference GPU build's call pattern (ProxyStep)
    against this library's FP64 matvec on the same inputs: result agreement, time per matvec
    and per step."""
    import numpy as np
    import torch
    from tensortoolkit_gb300 import workloads
    from tensortoolkit_gb300.api import ContractionPlan, DTensor, Matvec
    tensors = workloads.heisenberg(WORKLOAD["D"], WORKLOAD["qmax"], WORKLOAD["sigma"], WORKLOAD["seed"])
    lenv, psi, mpo1, mpo2, renv = tensors
    dl, dp, d1, d2, dr = (DTensor.from_host(x, local) for x in tensors)
    axes = [[[0], [0]], [[0, 2], [0, 1]], [[4, 1], [0, 1]], [[4, 1], [1, 0]]]
    steps, bufs, a_meta, a_buf = [], [], lenv, dl.buf
    for i, b in enumerate((dp, d1, d2, dr)):
        plan = ContractionPlan(a_meta, b.meta, axes[i], local)
        steps.append(ProxyStep(a_meta, b.meta, axes[i], plan))
        c = torch.zeros(max(plan.result.size, 1), dtype=torch.float64, device=f"cuda:{local}")
        bufs.append((a_buf, b.buf, c))
        a_meta, a_buf = plan.result, c
        del plan

    def proxy_matvec():
        for st, (a, b, c) in zip(steps, bufs):
            st.run(a, b, c)
    proxy_matvec()
    torch.cuda.synchronize()
    mv = Matvec(dl, psi, d1, d2, dr, mode="fp64")
    ours = mv.apply(dp).to_host()
    got = bufs[-1][2][: ours.size].cpu().numpy()
    err = float(np.linalg.norm(got - ours.data) / np.linalg.norm(ours.data))
    t_proxy = _time_events(proxy_matvec, stream, flush, reps=reps)
    # the same launches captured once into a CUDA graph and replayed: kernels only, without the
    # host's per-call dispatch (a lower bound for the pattern however it is issued)
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(device=f"cuda:{local}")
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        proxy_matvec()
    torch.cuda.current_stream().wait_stream(side)
    with torch.cuda.graph(graph):
        proxy_matvec()
    bufs[-1][2].zero_()
    graph.replay()
    torch.cuda.synchronize()
    got_g = bufs[-1][2][: ours.size].cpu().numpy()
    err_g = float(np.linalg.norm(got_g - ours.data) / np.linalg.norm(ours.data))
    t_graph = _time_events(graph.replay, stream, flush, reps=reps)
    per_step = []
    for st, (a, b, c) in zip(steps, bufs):
        per_step.append(round(_time_events(lambda: st.run(a, b, c), stream, flush, reps=reps), 3))
    o = DTensor.empty(mv.result, local)
    t_ours = _time_events(lambda: mv.apply(dp, o), stream, flush, reps=10)
    ntasks = sum(len(st.tasks) for st in steps)
    return {"proxy_fp64_ms_per_matvec": round(t_proxy, 3), "proxy_ms_per_step": per_step,
            "proxy_graph_ms_per_matvec": round(t_graph, 3), "proxy_graph_vs_ours_rel_err": err_g,
            "ours_fp64_ms_per_matvec": round(t_ours, 4), "ours_vs_proxy_speedup": round(t_proxy / t_ours, 2),
            "ours_vs_proxy_graph_speedup": round(t_graph / t_ours, 2),
            "proxy_vs_ours_rel_err": err, "gemm_calls_per_matvec": ntasks,
            "note": "labelled proxy of the reference CUDA build's pattern (the build itself needs cuTENSOR, "
                    "absent on this host): per operand block one strided-copy permute, then one cuBLAS "
                    "DGEMM per task in task order on one stream, with torch's caching allocator in place "
                    "of the reference's cudaMalloc / cudaFree per transposed block (so the proxy is, if "
                    "anything, faster than the reference build); proxy_graph = the same launches "
                    "replayed from one CUDA graph (no per-call host dispatch: a lower bound)"}


def run_adapter_costs(local: int) -> dict:
    """What one qlten_gb300::Contract costs a caller at D=4000, by the C-ABI calls the adapter
    makes (device buffers, as in a GPU build of qlten): a first call creates the plan (device
    sector pairing, task list, transposes' work lists), tunes its schedule and executes; a
    later call with the same layouts finds the plan in the context's cache and only executes.
    Wall time on the host, the device synchronised at the end of each call."""
    import torch
    from tensortoolkit_gb300 import workloads
    from tensortoolkit_gb300.api import ContractionPlan, DTensor, Contract
    tensors = workloads.heisenberg(WORKLOAD["D"], WORKLOAD["qmax"], WORKLOAD["sigma"], WORKLOAD["seed"])
    lenv, psi, mpo1, mpo2, renv = tensors
    dl, dp, dr = (DTensor.from_host(x, local) for x in (lenv, psi, renv))
    t1 = Contract(dl, dp, [[0], [0]])
    t2 = Contract(t1, DTensor.from_host(mpo1, local), [[0, 2], [0, 1]])
    t3 = Contract(t2, DTensor.from_host(mpo2, local), [[4, 1], [0, 1]])
    out = {}
    for name, a, b, axes in (("L.psi (step 0)", dl, dp, [[0], [0]]), ("t3.R (step 3)", t3, dr, [[4, 1], [1, 0]])):
        row = {}
        for mode in ("fp64", "split"):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            plan = ContractionPlan(a.meta, b.meta, axes, local)
            t_plan = time.perf_counter() - t0
            c = DTensor.empty(plan.result, local)
            t0 = time.perf_counter()
            plan.tune(a, b, c, mode=mode)
            t_tune = time.perf_counter() - t0
            t0 = time.perf_counter()
            plan.execute(a, b, c, mode=mode)
            torch.cuda.synchronize()
            t_first = time.perf_counter() - t0
            ts = []
            for _ in range(5):
                t0 = time.perf_counter()
                plan.execute(a, b, c, mode=mode)
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            plan.device_status()
            row[mode] = {"plan_create_ms": round(t_plan * 1e3, 3), "tune_ms": round(t_tune * 1e3, 3),
                         "first_exec_ms": round(t_first * 1e3, 3),
                         "cached_call_ms": round(statistics.median(ts) * 1e3, 3),
                         "schedule": {k: v for k, v in plan.schedule().items() if k != "tuned_ms"}}
            del plan, c
        out[name] = row
    out["note"] = ("C-ABI calls of the adapter's Contract: first call = plan create + tune + execute; cached call = "
                   "execute on the context's cached plan (result topology export and the qlten-side block "
                   "insertion are host bookkeeping not timed here)")
    return out


def run_profile_case(case: str, tensors, dev, local: int) -> None:
    """Profiling drivers (one small, fixed piece of work each, for ncu captures): the split GEMM
    of the D=4000 matvec's first (step0) or last (step3) contraction, stacked schedule, run
    twice; three applies of the Config 5 split matvec (fU(1) x U(1) complex, D=6000); Config 3's
    batched SVD; the stress QR (41 square blocks 10..800); the three batched permutes of t0
    (D=4000, 80 MB) measured by --aux, one launch each after t0 is made."""
    import torch
    from tensortoolkit_gb300 import workloads
    from tensortoolkit_gb300.api import Contract, ContractionPlan, DTensor, QR, SVD, TransposePlan
    lenv, psi, mpo1, mpo2, renv = tensors
    dl, dp, d1, d2, dr = dev
    if case == "permute":
        t0 = Contract(dl, dp, [[0], [0]])
        plans = [TransposePlan(t0.meta, perm, local) for perm in ((1, 3, 4, 0, 2), (4, 3, 2, 1, 0), (1, 0, 4, 2, 3))]
        outs = [DTensor.empty(pl.result, local) for pl in plans]
        torch.cuda.synchronize()
        for pl, o in zip(plans, outs):
            pl.execute(t0, o)
        torch.cuda.synchronize()
        print(json.dumps({"profile_run": True, "case": case}))
        return
    if case in ("step0", "step3"):
        if case == "step0":
            p, a, b = ContractionPlan(lenv, psi, [[0], [0]], local), dl, dp
        else:
            t1 = Contract(dl, dp, [[0], [0]])
            t2 = Contract(t1, d1, [[0, 2], [0, 1]])
            t3 = Contract(t2, d2, [[4, 1], [0, 1]])
            p, a, b = ContractionPlan(t3.meta, renv, [[4, 1], [1, 0]], local), t3, dr
        p.set_schedule(split_stack=1)
        c = DTensor.empty(p.result, local)
        for _ in range(2):
            p.execute(a, b, c, mode="split")
        torch.cuda.synchronize()
        p.device_status()
    elif case == "matvec5":
        from tensortoolkit_gb300.api import Matvec
        lenv5, psi5, m15, m25, renv5 = workloads.hubbard(6000, 10, 4)
        d5 = [DTensor.from_host(x, local) for x in (lenv5, psi5, m15, m25, renv5)]
        mv = Matvec(d5[0], psi5, d5[2], d5[3], d5[4], mode="split")
        o = DTensor.empty(mv.result, local)
        for _ in range(3):
            mv.apply(d5[1], o)
        torch.cuda.synchronize()
        mv.device_status()
        print(json.dumps({"mpo_form": mv.mpo_form()}))
    elif case == "svd":
        SVD(DTensor.from_host(workloads.svd_psi(2000, 20, 6.0, 3), local), 2, [0], 1e-9, 1, 2000)
    else:
        QR(DTensor.from_host(workloads.svd_stress(41, 10, 800, 3), local), 1, [0])
    torch.cuda.synchronize()
    print(json.dumps({"profile_run": True, "case": case}))


def run_aux(local: int, part: str = "all"):
    """Measurements beside the headline: the batched permute's achieved HBM bandwidth, the
    batched block SVD / QR (Config 3) against a per-block cuSOLVER loop on the same shapes
    (the reference GPU build's pattern), and the matvec of Configs 2 and 5."""
    import numpy as np
    import torch
    from tensortoolkit_gb300 import workloads
    from tensortoolkit_gb300.api import Contract, DTensor, Lanczos, Matvec, QR, SVD, Transpose, TransposePlan
    pk = peaks()
    out = {"aux": True, "gpu": torch.cuda.get_device_name(local)}
    dev = f"cuda:{local}"
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(local)
    # 1. permute: t0 of the D=4000 matvec (80 MB) to the order a contraction over its legs
    #    (0, 2) would use; every block moves (Transpose copies identity layouts too)
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(WORKLOAD["D"], WORKLOAD["qmax"], WORKLOAD["sigma"],
                                                       WORKLOAD["seed"])
    t0 = Contract(DTensor.from_host(lenv, local), DTensor.from_host(psi, local), [[0], [0]])
    for name, perm in () if part not in ("all", "transpose") else (("t0 (w,l,p1,p2,r) -> (l,p2,r,w,p1)", (1, 3, 4, 0, 2)),
                       ("t0 (w,l,p1,p2,r) -> (r,p2,p1,l,w)", (4, 3, 2, 1, 0)),
                       ("t0 (w,l,p1,p2,r) -> (l,w,r,p1,p2)", (1, 0, 4, 2, 3))):
        plan = TransposePlan(t0.meta, perm, local)
        dst = DTensor.empty(plan.result, local)
        plan.execute(t0, dst)
        ms = _time_events(lambda: plan.execute(t0, dst), stream, flush)
        ms_api = _time_events(lambda: Transpose(t0, perm), stream, flush)
        # the same launch after a flush that leaves L2 clean (write > L2, then read 256 MiB):
        # the write flush leaves L2 full of dirty lines whose write-back the next kernel pays
        clean = []
        for r in range(5):
            flush.fill_(float(r))
            flush[: flush.numel() // 2].sum()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.execute(t0, dst)
            e1.record(stream)
            clean.append((e0, e1))
        torch.cuda.synchronize()
        ms_clean = statistics.median(a.elapsed_time(b) for a, b in clean)
        nbytes = 2 * 8 * t0.meta.size
        out.setdefault("transpose", []).append(
            {"case": name, "mbytes_moved": nbytes / 1e6, "kernel_ms": round(ms, 4),
             "kernel_ms_clean_l2": round(ms_clean, 4),
             "frac_of_hbm_clean_l2": nbytes / (ms_clean / 1e3) / 1e9 / pk["hbm_gbs"],
             "gbs": nbytes / (ms / 1e3) / 1e9, "frac_of_hbm": nbytes / (ms / 1e3) / 1e9 / pk["hbm_gbs"],
             "api_call_ms": round(ms_api, 4),
             "note": "kernel_ms: qltg_transpose_plan_exec (one launch); api_call_ms: qltg_transpose, which "
                     "also builds and uploads the block list"})
        del dst, plan
    del t0
    # 2. batched SVD / QR (Config 3 and the 41-block stress variant) vs per-block cuSOLVER
    svd_cases = (("Config 3: psi D=2000, 41 block-matrices", workloads.svd_psi(2000, 20, 6.0, 3), 2),
                 ("stress: 41 square blocks 10..800", workloads.svd_stress(41, 10, 800, 3), 1))
    for name, t, ldims in svd_cases if part in ("all", "svd") else ():
        dt = DTensor.from_host(t, local)
        sv = time_call(lambda: SVD(dt, ldims, [0], 1e-9, 1, 2000))
        qr = time_call(lambda: QR(dt, ldims, [0]))
        shapes = svd_group_shapes(t, ldims)
        mats = [torch.randn(r, c, dtype=torch.float64, device=dev) for r, c in shapes]
        loop = time_call(lambda: [torch.linalg.svd(m, full_matrices=False) for m in mats])
        qloop = time_call(lambda: [torch.linalg.qr(m) for m in mats])
        out.setdefault("svd", []).append(
            {"case": name, "groups": len(shapes), "max_rows": max(r for r, _ in shapes),
             "max_cols": max(c for _, c in shapes), "batched_svd_ms": sv * 1e3,
             "per_block_cusolver_svd_ms": loop * 1e3, "batched_qr_ms": qr * 1e3,
             "per_block_cusolver_qr_ms": qloop * 1e3,
             "note": "batched = the whole qltg_svd / qltg_qr call (grouping, kernels, truncation, U/S/Vt "
                     "or Q/R tensors); per-block = torch.linalg.svd / qr (cuSOLVER) on dense matrices of "
                     "the same shapes, kernels only"})
        del dt, mats
    # 3. matvec of Config 2 (U(1), D=2000) and Config 5 (fermionic complex128, D=6000), each in
    #    plain FP64 and split precision
    def mv_time(tensors, mode, lanczos_steps=0):
        lenv_, psi_, mpo1_, mpo2_, renv_ = tensors
        dl_, dp_, d1_, d2_, dr_ = (DTensor.from_host(x, local) for x in tensors)
        t_create = time.perf_counter()
        mv = Matvec(dl_, psi_, d1_, d2_, dr_, mode=mode)
        torch.cuda.synchronize()
        t_create = time.perf_counter() - t_create
        o = DTensor.empty(mv.result, local)
        ms = _time_events(lambda: mv.apply(dp_, o), stream, flush, reps=10)
        mv.device_status()
        f, _ = mv.stats()
        # 8(d): P = FP64 pipe (fp64) or BF16 peak / 28 slice products (split), BW = HBM
        peak = fp64_peak_tflops(local, stream) if mode == "fp64" else pk["bf16_tflops"] / 28.0
        _, t_bound = matvec_step_bounds(tensors, local, peak, pk["hbm_gbs"])
        r = {"mode": mode, "ms": round(ms, 4), "gflops": f / (ms / 1e3) / 1e9, "plan_s": round(t_create, 3),
             "schedules": mv.schedules(),
             "gflop_per_matvec": round(f / 1e9, 4), "peak_tflops": round(peak, 2),
             "sum_T_bound_ms": round(t_bound, 4), "frac_sum_T_over_t": round(t_bound / ms, 4)}
        if lanczos_steps:
            # the graph-captured Lanczos: one CUDA graph per step (matvec + two-pass complex
            # Gram-Schmidt + norm); steps captured on a first run, then timed from a restart
            lz = Lanczos(mv, lanczos_steps)
            lz.start(dp_)
            lz.step(lanczos_steps)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            flush.fill_(1.0)
            lz.start(dp_)
            e0.record(stream)
            lz.step(lanczos_steps)
            e1.record(stream)
            torch.cuda.synchronize()
            a, b = lz.coeffs()
            mv.device_status()
            lms = e0.elapsed_time(e1)
            r["lanczos"] = {"steps": lanczos_steps, "total_ms": round(lms, 3),
                            "ms_per_step": round(lms / lanczos_steps, 4),
                            "lowest_ritz": float(Lanczos.ritz_lowest(a, b)[-1]),
                            "note": "random complex operands: H is not Hermitian, the Ritz value is the "
                                    "tridiagonal's lowest eigenvalue of the recurrence"}
            del lz
        del mv
        return r
    if part in ("all", "proxy"):
        out["fp64_vs_reference_gpu_pattern_d4000"] = run_proxy(local, stream, flush)
    if part in ("all", "fp64rates"):
        import ctypes as C
        from tensortoolkit_gb300 import capi
        from tensortoolkit_gb300.api import context, stream_ptr
        f, m = C.c_double(), C.c_double()
        capi.check(capi.lib().qltg_selftest_fp64_rates(context(local).h, C.byref(f), C.byref(m), stream_ptr(local)))
        out["fp64_rates"] = {"dfma_tflops": round(f.value, 3), "dmma_mma_sync_m8n8k4_tflops": round(m.value, 3),
                             "cublas_dgemm_8192_tflops": round(fp64_peak_tflops(local, stream), 3),
                             "note": "qltg_selftest_fp64_rates: DFMA loop (8 chains per thread) and mma.sync "
                                     "m8n8k4 f64 loop (4 fragments per warp, 512 flops each) over 8 CTAs per SM"}
    if part in ("all", "adapter"):
        out["adapter_contract_costs_d4000"] = run_adapter_costs(local)
    if part in ("all", "matvec"):
        c2 = workloads.heisenberg(2000, 20, 6.0, 1)
        out["config2_matvec_d2000"] = [mv_time(c2, "fp64"), mv_time(c2, "split")]
        c5 = workloads.hubbard(6000, 10, 4)
        out["config5_matvec_d6000_complex"] = [mv_time(c5, "fp64", 20), mv_time(c5, "split", 20)]
    print(json.dumps(out))


def cpu_matvec_time(tensors, iters: int, threads: int) -> float:
    """Seconds per matvec of the CPU restatement (median of `iters` after one warm-up)."""
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


def cpu_thread_sweep(tensors, iters: int = 3):
    """The CPU restatement at 1, 2, 4 and all host threads (the reference's default is 4:
    framework/consts.h:24, framework/hp_numeric/omp_set.h:27-83). Returns ({threads: s/iter},
    best thread count)."""
    n = os.cpu_count() or 1
    counts = sorted({1, 2, 4, n} & set(range(1, n + 1)))
    sweep = {t: cpu_matvec_time(tensors, iters, t) for t in counts}
    return sweep, min(sweep, key=sweep.get)


def run_reference(args):
    """The reference's algorithm on the host cores: the CPU restatement (oracle/oracle.cc,
    OpenBLAS dgemm per block pair as the reference's CPU build) on the same synthetic D=4000
    inputs, made by the generator compiled into the oracle's own library. A short thread
    sweep picks the thread count; the timed steps run at the best one."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    from oracle import oracle
    tensors = oracle.workload("matvec_u1", WORKLOAD["qmax"], WORKLOAD["sigma"], WORKLOAD["D"], WORKLOAD["seed"])
    sweep, threads = cpu_thread_sweep(tensors)
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
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded N(0,1) operands with the reference case's shapes)",
           "config": bench_config(world), "impl": "reference",
           "cpu_baseline": {"value": v, "unit": "s/iter", "cores": threads, "kind": "port",
                            "sample": f"{args.steps} full D=4000 matvecs after {args.warmup} warm-up, at the best "
                                      f"thread count of the sweep",
                            "cpu_model": cpu_model(), "nproc": os.cpu_count(),
                            "thread_sweep_s_per_iter": {str(k): round(x, 4) for k, x in sweep.items()},
                            "reference_default_threads": 4,
                            "at_default_threads_s_per_iter": round(sweep.get(4, float("nan")), 4)},
           "e2e": {"value": v, "unit": "s/iter", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["both", "split", "fp64"], default=os.environ.get("QLTG_BENCH_MODE", "both"),
                    help="both (default): headline split precision, plain FP64 beside it")
    ap.add_argument("--cpu-iters", type=int, default=None, help="CPU baseline sample size")
    ap.add_argument("--aux", action="store_true",
                    help="measurements beside the headline: permute GB/s, batched SVD/QR vs per-block, "
                         "Config 2 and Config 5 matvecs (one JSON line)")
    ap.add_argument("--aux-part", choices=["all", "transpose", "svd", "matvec", "proxy", "adapter", "fp64rates"], default="all")
    ap.add_argument("--profile", action="store_true",
                    help="profiling run: plan the D=4000 matvec, apply it twice, print nothing else")
    ap.add_argument("--profile-case", choices=["matvec", "matvec5", "step0", "step3", "svd", "qr", "permute"], default="matvec",
                    help="with --profile: the matvec (default); one of its split-precision GEMM steps "
                         "(stacked schedule, executed twice); Config 3's batched SVD; the stress QR")
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
    stream = torch.cuda.current_stream(local)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")
    modes = ["split", "fp64"] if args.mode == "both" else [args.mode]

    if args.aux:
        return run_aux(local, args.aux_part)

    if args.profile and args.profile_case != "matvec":
        return run_profile_case(args.profile_case, tensors, (dl, dp, d1, d2, dr), local)

    if args.profile:
        for m in modes:
            mv = Matvec(dl, psi, d1, d2, dr, mode=m)
            out = DTensor.empty(mv.result, local)
            for _ in range(2):
                mv.apply(dp, out)
            torch.cuda.synchronize()
        print(json.dumps({"profile_run": True, "modes": modes}))
        return

    pk = peaks()
    results = {}
    clk_summary = None
    for m in modes:
        mv = Matvec(dl, psi, d1, d2, dr, mode=m)
        flops, launches_per_step = mv.stats()
        out = DTensor.empty(mv.result, local)
        for _ in range(args.warmup):
            mv.apply(dp, out)
        torch.cuda.synchronize()
        mv.device_status()
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
        mv.device_status()
        t_step = sum(a.elapsed_time(b) for a, b in evs) / 1e3 / args.steps
        if clk_summary is None:
            clk_summary = clk.summary()
        # end to end through the public API with pinned host buffers
        # (qltg_matvec_apply_host: psi copied in, the product, the result copied out)
        h_in = torch.from_numpy(psi.raw_f64()).pin_memory()
        h_out = torch.empty(mv.result.size, dtype=torch.float64).pin_memory()
        for _ in range(2):
            mv.apply_host(h_in, h_out)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.steps):
            mv.apply_host(h_in, h_out)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_step = e0.elapsed_time(e1) / 1e3 / args.steps
        roof = gemm_roofline(m, lenv, psi, d1, d2, dr, dl, dp, local, stream, flush, pk)
        roof["sum_T_over_t"] = roof["sum_T_bound_ms"] / (t_step * 1e3)
        results[m] = {"s_per_iter": t_step, "e2e_s_per_iter": e2e_step, "flops": flops,
                      "launches_per_step": launches_per_step, "roofline": roof, "schedules": mv.schedules(),
                      "h2d": int(h_in.numel() * 8), "d2h": int(h_out.numel() * 8)}
        del mv, out

    head = results[modes[0]]
    t_step = head["s_per_iter"]
    # max over ranks
    t_max = replica_time(t_step, world, f"cuda:{local}")

    if rank == 0:
        cpu = None
        try:
            cpu_iters = 10 if args.cpu_iters is None else args.cpu_iters
            sweep, threads = cpu_thread_sweep(tensors)
            v = cpu_matvec_time(tensors, cpu_iters, threads)
            cpu = {"value": v, "unit": "s/iter", "cores": threads, "kind": "port",
                   "sample": f"median of {cpu_iters} full D=4000 matvecs (OpenBLAS dgemm per block pair) at the "
                             f"best thread count of the sweep",
                   "cpu_model": cpu_model(), "nproc": os.cpu_count(),
                   "thread_sweep_s_per_iter": {str(k): round(x, 4) for k, x in sweep.items()},
                   "at_default_threads_s_per_iter": round(sweep.get(4, float("nan")), 4)}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "s/iter", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"unavailable: {e}"}
        res = {
            "metric": METRIC, "value": t_max / world, "unit": "s/iter", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "precision": ("split: FP64 emulated with BF16 slices on tcgen05, <=1e-12 rel. err vs FP64"
                          if modes[0] == "split" else "plain FP64"),
            "data": "synthetic (seeded N(0,1) operands with the reference case's shapes)",
            "config": bench_config(world),
            "mode": modes[0],
            "gflops_fp64_equiv": head["flops"] / t_step / 1e9,
            "algorithmic_gflop_per_step": head["flops"] / 1e9,
            "e2e": {"value": head["e2e_s_per_iter"], "unit": "s/iter", "h2d_bytes_per_step": head["h2d"],
                    "d2h_bytes_per_step": head["d2h"]},
            "gpu_launches": int(head["launches_per_step"] * args.steps),
            "gpu_launches_per_step": int(head["launches_per_step"]),
            "roofline": head["roofline"],
            "tuned_schedules": head["schedules"],
            "cpu_baseline": cpu,
            "clocks": clk_summary,
        }
        if len(modes) > 1:
            f = results["fp64"]
            res["fp64"] = {"s_per_iter": f["s_per_iter"], "e2e_s_per_iter": f["e2e_s_per_iter"],
                           "roofline": f["roofline"], "gpu_launches_per_step": int(f["launches_per_step"]),
                           "tuned_schedules": f["schedules"]}
            res["split_speedup_vs_fp64"] = f["s_per_iter"] / head["s_per_iter"]
            res["precision_study"] = precision_study(local)
        print(json.dumps(res))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
