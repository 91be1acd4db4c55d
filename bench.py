"""Benchmark of PDL's broadcast-loop hot path on GB300.

Headline (one JSON line on rank 0): Ufunc reduction GB/s over dim 0 of the
float64 (4096, 2048) ndarray, uniform[-1,1) from seed 1, no bad values: one
step = sumover, prodover, average, minimum, maximum, minimum_ind and
cumusumover, each reading its own one of 6 device copies of the input (384
MiB in rotation, more than twice the 129 MB L2, so every op streams from
HBM).  value = algorithmic bytes (inputs read once + outputs written once)
/ device time (CUDA events on the library's stream).  e2e = the same ops
through the C ABI starting from pinned host memory: the step copies the
input to its device mirror, runs the seven ops and copies every result back.

The same line carries the float32 matmult measurement (a(t=1024,h=2048)
batch 16 x b(w=2048,t=1024), N(0,1)): TFLOP/s of the split-bf16 tensor-core
kernel and of the plain FP32 SIMT kernel, each with its max normwise error
against an FP64 product on sampled rows.

--impl reference times the reference's algorithm on the host cores (the C
restatement of the reference loops, with the reference's auto-pthread
split over all host threads) on the same workload and metric.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

UFUNC_OPS = ["sumover", "prodover", "average", "minimum", "maximum", "minimum_ind",
             "cumusumover"]
N0, N1 = 4096, 2048            # PDL dims (n, rows)
NCOPIES = 6
METRIC = "Ufunc reduce GB/s over dim 0 (sumover, prodover, average, minimum, maximum, minimum_ind, cumusumover)"
WORKLOAD = "PDL::Ufunc family over dim 0 of float64 ndarray dims (4096,2048), uniform[-1,1) seed 1, no bad values"
# dram__bytes_read.sum + dram__bytes_write.sum of one sumover launch on this
# workload, from the ncu capture summarised in profiles/ (None: not captured)
NCU_TRAFFIC_SUMOVER = None


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def c1_input():
    rng = np.random.default_rng(1)
    return rng.uniform(-1.0, 1.0, size=(N1, N0))  # numpy order: PDL dims (4096, 2048)


def op_bytes(op):
    inb = N0 * N1 * 8
    if op == "cumusumover":
        return inb * 2
    return inb + N1 * 8


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, gpu_index=0):
        self.proc = None
        self.out = None
        self.idx = gpu_index

    def __enter__(self):
        try:
            self.out = open(ROOT / "gpurun_out" / "bench_clocks.csv", "w") if (ROOT / "gpurun_out").exists() \
                else open(os.devnull, "w")
            self.tmp = []
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}",
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.lines = []
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.th.join(timeout=2)
        if self.out:
            self.out.write("\n".join(getattr(self, "lines", [])))
            self.out.close()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- our arm

def run_ours(args, rank, world):
    import torch

    import pdl_gb300 as P
    from pdl_gb300 import _abi as A

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    P.set_stream(stream.cuda_stream)
    hbm, bf16, peak_kind = peaks()

    host = c1_input()
    copies = []
    for _ in range(NCOPIES):
        x = P.pdl(host)
        x.to_device()
        x.storage.host = None  # device-resident only
        x.storage.fresh = "dev"
        copies.append(x)
    outs = {}
    for op in UFUNC_OPS:
        r = getattr(P, op)(copies[0])
        outs[op] = r  # device-resident preallocated outputs of the right shape/type
    P.sync()

    def step(k, times=None, ev=None):
        launches = 0
        for j, op in enumerate(UFUNC_OPS):
            x = copies[(k * len(UFUNC_OPS) + j) % NCOPIES]
            if ev is not None:
                ev[j][0].record(stream)
            getattr(P, op)(x, outs[op])
            if ev is not None:
                ev[j][1].record(stream)
            launches += P.last_launch_info()["nlaunches"]
        return launches

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    # per-op device times (events around each op), then the whole K-step region
    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in UFUNC_OPS] for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    launches = 0
    with Clocks(dev.index) as clk:
        # keep the GPU busy while the host enqueues the timed ops, so the
        # events time back-to-back kernels, not host launch overhead
        torch.cuda._sleep(int(2.0e9 * 0.06))
        t0.record(stream)
        for k in range(args.steps):
            launches += step(k, ev=ev[k])
        t1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    total_ms = t0.elapsed_time(t1)
    per_op = {op: [ev[k][j][0].elapsed_time(ev[k][j][1]) for k in range(args.steps)]
              for j, op in enumerate(UFUNC_OPS)}
    step_bytes = sum(op_bytes(op) for op in UFUNC_OPS)
    kernel_ms = sum(sum(v) for v in per_op.values()) / args.steps
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * step_bytes / (ms_per_step * 1e-3) / 1e9
    op_gbs = {op: op_bytes(op) / (statistics.mean(v) * 1e-3) / 1e9 for op, v in per_op.items()}
    op_ms = {op: statistics.mean(v) for op, v in per_op.items()}
    dominant = max(op_ms, key=op_ms.get)

    # -------- e2e: host (pinned) -> device mirror -> the ops -> results to host
    e2e = run_e2e(args, P, A, torch, host, copies, outs, step_bytes, world) if args.e2e else None

    result = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded numpy uniform[-1,1))",
        "config": {"workload": WORKLOAD, "ops_per_step": UFUNC_OPS,
                   "l2": f"inputs rotate over {NCOPIES} device copies "
                         f"({NCOPIES * N0 * N1 * 8 >> 20} MiB > 2x L2)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "per_op_gbs": op_gbs, "per_op_ms": op_ms, "kernel_ms_per_step": kernel_ms,
        "roofline": {"bound": "hbm", "kernel": dominant,
                     "achieved": op_gbs[dominant], "peak": hbm, "unit": "GB/s",
                     "frac": op_gbs[dominant] / hbm, "peak_kind": peak_kind,
                     "traffic": NCU_TRAFFIC_SUMOVER if dominant == "sumover" else None,
                     "family_frac": value / world / hbm},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if args.matmult and rank == 0:
        result["matmult"] = bench_matmult(args, P, torch, stream, bf16, peak_kind)
    if rank == 0 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(args, host)
    return result


def run_e2e(args, P, A, torch, host, copies, outs, step_bytes, world):
    """Through the C ABI from pinned host memory: copy the input to its
    device mirror, run the ops, copy every result back; wall time per step."""
    pinned_in = torch.empty(N0 * N1, dtype=torch.float64, pin_memory=True)
    pinned_in.numpy()[:] = host.reshape(-1)
    out_host = {op: torch.empty(outs[op].storage.nbytes, dtype=torch.uint8, pin_memory=True)
                for op in UFUNC_OPS}
    mirror = copies[0].storage.dev
    nbytes_in = N0 * N1 * 8
    L = A.lib()

    def e2e_step():
        A.check(L.pdlgb300_to_device(mirror, pinned_in.data_ptr(), nbytes_in))
        for op in UFUNC_OPS:
            getattr(P, op)(copies[0], outs[op])
        for op in UFUNC_OPS:
            A.check(L.pdlgb300_to_host(out_host[op].data_ptr(), outs[op].storage.dev,
                                       outs[op].storage.nbytes))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - te) * 1e3 / args.steps
    d2h = sum(outs[op].storage.nbytes for op in UFUNC_OPS)
    return {"value": world * step_bytes / (e2e_ms * 1e-3) / 1e9, "unit": "GB/s",
            "h2d_bytes_per_step": nbytes_in, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms}


def bench_matmult(args, P, torch, stream, bf16, peak_kind):
    rng = np.random.default_rng(4)
    T, H, W, NB = 1024, 2048, 2048, args.mm_batch
    a = rng.standard_normal((NB, H, T)).astype(np.float32)   # PDL dims (t, h, batch)
    b = rng.standard_normal((T, W)).astype(np.float32)       # PDL dims (w, t)
    x = P.pdl(a).to_device()
    y = P.pdl(b).to_device()
    flops = 2.0 * T * H * W * NB
    out = {}
    rows = rng.choice(H, size=32, replace=False)
    zs = rng.choice(NB, size=min(NB, 2), replace=False)
    for name, mode in [("bf16x6", P.MATMULT_BF16X6), ("bf16x3", P.MATMULT_BF16X3),
                       ("simt_fp32", P.MATMULT_SIMT_FP32)]:
        P.set_matmult_mode(mode)
        c = P.matmult(x, y)
        P.sync()
        kern = P.last_launch_info()["kernel"]
        ts = []
        for _ in range(args.mm_steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            P.matmult(x, y, c)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        ms = statistics.median(ts)
        cn = c.numpy()
        err = 0.0
        for z in zs:
            ref = a[z][rows].astype(np.float64) @ b.astype(np.float64)
            err = max(err, float(np.max(np.abs(cn[z][rows] - ref)) / np.max(np.abs(ref))))
        out[name] = {"tflops": flops / (ms * 1e-3) / 1e12, "ms": ms, "kernel": kern,
                     "max_normwise_rel_err": err}
    P.set_matmult_mode(P.MATMULT_BF16X6)
    out["config"] = f"a(t=1024,h=2048) x b(w=2048,t=1024), batch {NB}, float32 N(0,1) seed 4"
    out["speedup_bf16x6_vs_simt"] = out["bf16x6"]["tflops"] / out["simt_fp32"]["tflops"]
    out["tensor_peak_tflops"] = bf16
    out["tensor_peak_kind"] = peak_kind
    return out


# ------------------------------------------------------------- CPU baseline

def cpu_time_family(host, nthreads, budget_s):
    """The oracle (the reference's loops in C with its pthread split) on the
    full workload, repeated until budget_s; returns GB/s and steps."""
    import pdl_gb300 as P  # host-only construction of descriptors
    from oracle import oracle as O
    x = P.pdl(host)
    step_bytes = sum(op_bytes(op) for op in UFUNC_OPS)
    steps, t0 = 0, time.perf_counter()
    while True:
        for op in UFUNC_OPS:
            O.run(op, [x], nthreads=nthreads)
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return steps * step_bytes / el / 1e9, steps, el


def cpu_baseline(args, host):
    n = os.cpu_count() or 1
    gbs, steps, el = cpu_time_family(host, n, args.cpu_budget)
    return {"value": gbs, "unit": "GB/s", "cores": n, "kind": "port",
            "sample": f"{steps} full steps of the 7-op family ({el:.1f} s), "
                      f"auto-pthread split over {n} threads"}


def run_reference(args, rank, world):
    host = c1_input()
    n = os.cpu_count() or 1
    gbs0, _, _ = cpu_time_family(host, n, 0.0)  # warm
    ts = []
    step_bytes = sum(op_bytes(op) for op in UFUNC_OPS)
    for _ in range(args.warmup):
        cpu_time_family(host, n, 0.0)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cpu_time_family(host, n, 0.0)
        ts.append(time.perf_counter() - t0)
    ms = statistics.mean(ts) * 1e3
    value = step_bytes / (ms * 1e-3) / 1e9
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy uniform[-1,1))",
            "config": {"workload": WORKLOAD, "ops_per_step": UFUNC_OPS},
            "cpu_baseline": {"value": value, "unit": "GB/s", "cores": n, "kind": "port",
                             "sample": "one full 7-op step per timed step, "
                                       f"auto-pthread split over {n} threads"},
            "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    global UFUNC_OPS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-matmult", dest="matmult", action="store_false")
    ap.add_argument("--mm-batch", type=int, default=16)
    ap.add_argument("--mm-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=8.0)
    ap.add_argument("--ops", default=",".join(UFUNC_OPS),
                    help="comma-separated subset of the Ufunc family (for profiling)")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    args = ap.parse_args()
    UFUNC_OPS = [o for o in args.ops.split(",") if o]
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, rank, world)))
        return 0
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    res = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(res))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
