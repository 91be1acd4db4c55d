"""Benchmark of PDL's broadcast-loop hot path on GB300.

Headline (one JSON line on rank 0): Ufunc reduce GB/s on the float32
accuracy-stress workload -- an ndarray of dims (65536, 4096) plus one row of
2^27 elements, magnitudes lognormal(0, 4) with random signs, 1% BAD (badflag
on), seeded: one step = sumover, average and cumusumover over dim 0 of both
(compensated float32 accumulation, the default).  Inputs (1.5 GiB) exceed
the 129 MB L2.  value = algorithmic bytes (inputs read once + outputs
written once) / device time (CUDA events on the library's stream, a GPU
sleep enqueued first so host launches run ahead).  e2e = the same ops
through the C ABI from pinned host memory: copy the inputs to their device
mirrors, run, copy every result back.

The same line carries: the accuracy of compensated vs plain float32 vs the
float64 path on that workload; the float64 (4096, 2048) Ufunc family
(sumover, prodover, average, minimum, maximum, minimum_ind, cumusumover on
6 rotating device copies, 384 MiB > 2x L2); and the float32 matmult
(a(t=1024,h=2048) batch 16 x b(w=2048,t=1024)): TFLOP/s of the split-bf16
tensor-core kernels and of the plain FP32 SIMT kernel with their max
normwise errors against FP64 on sampled rows.  Each of these per-op figures
is timed with CUDA events around one library call, with a 1 ms GPU sleep
enqueued before the start event, so that the host's planning and launch
latency is not counted as device time (the call's own synchronisation,
where it has one, still is).

--impl reference times the reference's algorithm on the host cores (the C
restatement of the reference loops, with the reference's auto-pthread split
over all host threads) on the same workload and metric, on a bounded
sample of rows.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(1, str(ROOT / "tests"))  # config_inputs: the configurations' seeded inputs

UFUNC_OPS = ["sumover", "prodover", "average", "minimum", "maximum", "minimum_ind",
             "cumusumover"]
C5_OPS = ["sumover", "average", "cumusumover"]
N0, N1 = 4096, 2048            # float64 family: PDL dims (n, rows)
NCOPIES = 6
C5_N, C5_ROWS, C5_LONG = 65536, 4096, 1 << 27
METRIC = "Ufunc reduce GB/s over dim 0 (sumover, average, cumusumover; compensated float32, 1% BAD)"
WORKLOAD = ("PDL::Ufunc sumover/average/cumusumover over dim 0 of float32 dims (65536,4096) "
            "plus one row of 2^27, lognormal(0,4) magnitudes with random sign, 1% BAD, seed 7")
FAMILY = "float64 dims (4096,2048) uniform[-1,1) seed 1, no bad values"
# dram__bytes_read.sum + dram__bytes_write.sum per launch of the dominant
# kernel on this workload, from the ncu captures summarised in profiles/
# (k_scan_rowblk captured at 3648 rows, scaled by 4096/3648 to the matrix;
# k_scan_chain on the 2^27 row as captured)
NCU_TRAFFIC = {"cumusumover[matrix]": (956.519168e6 + 924.768256e6) * 4096 / 3648,
               "cumusumover[row]": 537.38e6 + 476.43e6}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def c1_input():
    rng = np.random.default_rng(1)
    return rng.uniform(-1.0, 1.0, size=(N1, N0))  # numpy order: PDL dims (4096, 2048)


def c5_inputs(rows=None, long_row=True):
    """float32 (rows, n) matrix and one long row: lognormal(0, 4) magnitude,
    random sign, 1% set to float's default badvalue (-FLT_MAX); the seeded
    generator shared with the tests (the same bits on every platform)."""
    import config_inputs as CI
    d = CI.c5(rows=rows or C5_ROWS, long_n=C5_LONG if long_row else 0)
    return d["mat"], (d["row"].reshape(-1) if long_row else None)


def op_bytes(op, n=N0, rows=N1, isz=8, osz=8):
    if op.startswith("cumu") or op.startswith("dcumu"):
        return rows * n * (isz + osz)
    return rows * n * isz + rows * (8 if op.endswith("_ind") else osz)


FIXTURES = ROOT / "tests" / "golden" / "pdl_fixtures.npz"


def pdl_fixtures():
    """The reference PDL's own outputs on these seeded inputs (made by
    tests/golden/make_pdl_fixtures.py), or None."""
    try:
        return np.load(FIXTURES)
    except OSError:
        return None


def errs(got, want):
    """Max elementwise relative error (|want| the denominator; the absolute
    error where want is 0), normwise error, and whether the bits are equal.
    NaN positions must agree; BAD (NaN or badvalue) positions are compared as
    values."""
    got, want = np.ascontiguousarray(got), np.ascontiguousarray(want)
    exact = got.dtype == want.dtype and got.shape == want.shape and \
        np.array_equal(got.view(np.uint8), want.view(np.uint8))
    g, w = got.astype(np.float64), want.astype(np.float64)
    nan = np.isnan(g) & np.isnan(w)
    d = np.where(nan, 0.0, np.abs(g - w))
    den = np.abs(np.where(nan, 0.0, w))
    rel = np.where(den > 0, d / np.where(den > 0, den, 1.0), d)
    nw = float(np.linalg.norm(d.ravel()) / max(np.linalg.norm(den.ravel()), 1e-300))
    return {"max_rel_err": float(np.nanmax(rel)) if rel.size else 0.0, "normwise_err": nw,
            "bit_exact": bool(exact)}


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, gpu_index=0):
        self.proc = None
        self.idx = gpu_index
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}",
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            time.sleep(0.15)
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
        log = os.environ.get("PDLGB300_CLOCKS_LOG")
        if log:  # the raw samples, appended for the record
            with open(log, "a") as f:
                f.write("\n".join(self.lines) + "\n")

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
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


def max_over_ranks(torch, value, device):
    """The largest of every rank's value (each rank's device time): the job
    is as slow as its slowest replica."""
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def timed_steps(torch, stream, steps, warmup, one_step, nops):
    """Run warmup untimed steps, then `steps` timed ones with a GPU sleep
    enqueued first; returns total ms, per-op ms lists, launches, clocks."""
    for k in range(warmup):
        one_step(k, None)
    torch.cuda.synchronize()
    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(nops)] for _ in range(steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    launches = 0
    with Clocks(torch.cuda.current_device()) as clk:
        torch.cuda._sleep(int(2.0e9 * 0.05))
        t0.record(stream)
        for k in range(steps):
            launches += one_step(k, ev[k])
        t1.record(stream)
        torch.cuda.synchronize()
    total = t0.elapsed_time(t1)
    per_op = [[ev[k][j][0].elapsed_time(ev[k][j][1]) for k in range(steps)] for j in range(nops)]
    return total, per_op, launches, clk.summary()


# ------------------------------------------------------------- our arm

def run_ours(args, rank, world):
    import torch

    import pdl_gb300 as P
    from pdl_gb300 import _abi as A

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    P.set_stream(stream.cuda_stream)
    hbm, bf16, peak_kind = peaks()
    L = A.lib()

    # ---------------- headline: config 5, compensated float32 with BAD
    mat, row = c5_inputs(args.c5_rows)
    xs = []
    for arr in (mat, row):
        x = P.pdl(arr)
        x.badflag(1)
        x.to_device()
        xs.append(x)
    work = [(op, j) for op in args.c5_ops.split(",") for j in range(2)]
    outs = {(op, j): getattr(P, op)(xs[j]) for op, j in work}
    P.sync()
    shapes = [(C5_N, mat.shape[0]), (C5_LONG, 1)]
    wbytes = [op_bytes(op, *shapes[j], isz=4, osz=4) for op, j in work]

    def one_step(k, ev):
        n = 0
        for i, (op, j) in enumerate(work):
            if ev is not None:
                ev[i][0].record(stream)
            getattr(P, op)(xs[j], outs[(op, j)])
            if ev is not None:
                ev[i][1].record(stream)
            n += P.last_launch_info()["nlaunches"]
        return n

    if world > 1:
        torch.distributed.barrier()
    total, per_op, launches, clocks = timed_steps(torch, stream, args.steps, args.warmup,
                                                  one_step, len(work))
    if world > 1:
        torch.distributed.barrier()
        total = max_over_ranks(torch, total, dev)
    step_bytes = sum(wbytes)
    ms_per_step = total / args.steps
    value = world * step_bytes / (ms_per_step * 1e-3) / 1e9
    op_ms = {f"{op}[{'matrix' if j == 0 else 'row'}]": statistics.mean(per_op[i])
             for i, (op, j) in enumerate(work)}
    op_gbs = {k: wbytes[i] / (v * 1e-3) / 1e9 for i, (k, v) in enumerate(op_ms.items())}
    dom = max(op_ms, key=op_ms.get)
    result = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded numpy lognormal(0,4), random sign, 1% BAD)",
        "config": {"workload": WORKLOAD, "ops_per_step": [f"{op}[{'matrix' if j == 0 else 'row'}]"
                                                          for op, j in work],
                   "accumulation": "compensated float32 (default)",
                   "l2": "inputs 1.5 GiB > 129 MB L2 (no reuse between ops)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "per_op_gbs": op_gbs, "per_op_ms": op_ms,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": op_gbs[dom], "peak": hbm,
                     "unit": "GB/s", "frac": op_gbs[dom] / hbm, "peak_kind": peak_kind,
                     "traffic": NCU_TRAFFIC.get(dom), "step_frac": value / world / hbm},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if args.e2e:
        result["e2e"] = c5_e2e(args, P, A, torch, (mat, row), xs, outs, work, step_bytes, world)
    if rank == 0 and args.accuracy:
        result["accuracy"] = c5_accuracy(P, xs, (mat, row))
    del xs, outs
    torch.cuda.empty_cache()

    if rank == 0 and args.family:
        result["f64_family"] = run_family(args, P, torch, stream, hbm)
    if args.matmult and rank == 0:
        result["matmult"] = bench_matmult(args, P, torch, stream, bf16, peak_kind)
    if args.secondary and rank == 0:
        result["fused_c2"] = bench_c2(args, P, torch, stream)
        result["adjoint_c4"] = bench_c4(args, P, torch, stream)
        result["inner_c3"] = bench_inner(args, P, torch, stream, hbm)
        result["expr"] = bench_expr(args, P, torch, stream, hbm)
        result["sort"] = bench_sort(args, P, torch, stream, hbm)
        result["fastraw"] = bench_fastraw(args, P, torch, stream)
    if rank == 0 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(args, mat, row)
    return result


def c5_e2e(args, P, A, torch, arrays, xs, outs, work, step_bytes, world):
    """Through the C ABI from pinned host memory: every step copies both
    inputs to their device mirrors, runs the six ops and copies every result
    back to pinned host memory.  Steps are pipelined the way a caller of the
    async copy entry points would: two sets of device mirrors alternate,
    host-to-device copies run on one stream and device-to-host copies on
    another (the host link carries both directions at once), the ops on the
    library's stream, ordered by events (an op waits for its step's inputs
    and for the previous read-back of its output buffer; a result is read
    back as soon as its op is done)."""
    L = A.lib()
    pins = []
    for arr in arrays:
        t = torch.empty(arr.size, dtype=torch.float32, pin_memory=True)
        t.numpy()[:] = arr.reshape(-1)
        pins.append(t)
    outh = {k: torch.empty(o.storage.nbytes, dtype=torch.uint8, pin_memory=True)
            for k, o in outs.items()}
    xs_b = []
    for arr in arrays:
        x = P.pdl(arr)
        x.badflag(1)
        x.to_device()
        xs_b.append(x)
    outs_b = {(op, j): getattr(P, op)(xs_b[j]) for op, j in work}
    P.sync()
    sets = [(xs, outs), (xs_b, outs_b)]
    comp = torch.cuda.current_stream()
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    inputs_free = [None, None]               # comp: the set's last op done
    output_free = [dict(), dict()]           # s_out: the set's read-back done, per output

    def e2e_step(k):
        j = k % 2
        X, O = sets[j]
        if inputs_free[j] is not None:
            s_in.wait_event(inputs_free[j])
        h2d = []
        for i, x in enumerate(X):
            A.check(L.pdlgb300_to_device_async(x.storage.dev, pins[i].data_ptr(),
                                               x.storage.nbytes, s_in.cuda_stream))
            ev = torch.cuda.Event()
            ev.record(s_in)
            h2d.append(ev)
        waited = set()
        for op, jj in work:
            key = (op, jj)
            if jj not in waited:          # an op waits for its own input only
                comp.wait_event(h2d[jj])
                waited.add(jj)
            if key in output_free[j]:
                comp.wait_event(output_free[j][key])
            getattr(P, op)(X[jj], O[key])
            done = torch.cuda.Event()
            done.record(comp)
            s_out.wait_event(done)
            o = O[key]
            A.check(L.pdlgb300_to_host_async(outh[key].data_ptr(), o.storage.dev,
                                             o.storage.nbytes, s_out.cuda_stream))
            back = torch.cuda.Event()
            back.record(s_out)
            output_free[j][key] = back
        last = torch.cuda.Event()
        last.record(comp)
        inputs_free[j] = last

    for k in range(2):
        e2e_step(k)
    torch.cuda.synchronize()
    n = max(10, args.steps)
    te = time.perf_counter()
    for k in range(n):
        e2e_step(k)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - te) * 1e3 / n
    # the read-back of the last step equals the device result
    for key, o in outs.items() if (n - 1) % 2 == 0 else outs_b.items():
        got = outh[key].numpy()[:16].tobytes()
        want = o.numpy().reshape(-1).view(np.uint8)[:16].tobytes()
        assert got == want, f"e2e read-back of {key} differs from the device result"
    del xs_b, outs_b
    return {"value": world * step_bytes / (ms * 1e-3) / 1e9, "unit": "GB/s",
            "h2d_bytes_per_step": sum(x.storage.nbytes for x in xs),
            "d2h_bytes_per_step": sum(o.storage.nbytes for o in outs.values()),
            "ms_per_step": ms, "steps": n,
            "pipelining": "2 device sets; H2D and D2H on their own streams, ordered by events"}


def c5_accuracy(P, xs, arrays):
    """Max errors of compensated and plain float32 against the float64 path
    (dsumover, daverage, dcumusumover on the GPU), per row: relative
    |x - x64| / |x64| and normwise |x - x64| / sum|a|."""
    mat, row = arrays
    res = {}
    bad = np.float32(-3.4028234663852886e38)
    for op, dop in [("sumover", "dsumover"), ("average", "daverage")]:
        for j, x in enumerate(xs):
            ref = getattr(P, dop)(x).numpy().astype(np.float64)
            a = (mat if j == 0 else row.reshape(1, -1))
            scale = np.where(a == bad, 0, np.abs(a.astype(np.float64))).sum(-1)
            if op == "average":
                scale = scale / np.maximum((a != bad).sum(-1), 1)
            key = f"{op}[{'matrix' if j == 0 else 'row'}]"
            res[key] = {}
            for mode, comp in [("compensated", True), ("plain", False)]:
                P.set_compensated(comp)
                got = getattr(P, op)(x).numpy().astype(np.float64)
                P.set_compensated(True)
                err = np.abs(got - ref)
                res[key][mode] = {"max_rel_err": float(np.max(err / np.maximum(np.abs(ref), 1e-300))),
                                  "max_normwise_err": float(np.max(err / scale))}
    # running sums: 32 sampled rows of the matrix, and the long row
    rs = np.random.default_rng(0).choice(C5_ROWS, 32, replace=False)
    for j, x in enumerate(xs):
        ref = P.dcumusumover(x).numpy()
        ref = ref[rs] if j == 0 else ref.reshape(1, -1)
        a = mat[rs] if j == 0 else row.reshape(1, -1)
        good = a != bad
        scale = np.cumsum(np.where(good, np.abs(a.astype(np.float64)), 0), -1)
        key = f"cumusumover[{'matrix' if j == 0 else 'row'}]"
        res[key] = {}
        for mode, comp in [("compensated", True), ("plain", False)]:
            P.set_compensated(comp)
            got = P.cumusumover(x).numpy()
            P.set_compensated(True)
            got = got[rs] if j == 0 else got.reshape(1, -1)
            err = np.abs(got.astype(np.float64) - ref)[good]
            rel = err / np.maximum(np.abs(ref[good]), 1e-300)
            res[key][mode] = {"max_rel_err": float(rel.max()),
                              "max_normwise_err": float((err / np.maximum(scale[good], 1e-300)).max())}
    res["reference_point"] = "float64 GPU path (d-variants), itself checked against the CPU oracle in tests"
    fx = pdl_fixtures()
    if fx is not None and mat.shape[0] == 4096:
        vs = {}
        for j, x in enumerate(xs):
            nm = "c5m" if j == 0 else "c5r"
            where = "matrix" if j == 0 else "row"
            for op in ("sumover", "average", "dsumover", "daverage"):
                vs[f"{op}[{where}]"] = errs(getattr(P, op)(x).numpy().reshape(-1),
                                            fx[f"{nm}/{op}"].reshape(-1))
            got = P.cumusumover(x).numpy()
            got = got[::64, ::128] if j == 0 else got.reshape(1, -1)[:, ::65536]
            vs[f"cumusumover[{where}]"] = errs(got, fx[f"{nm}/cumusumover/sample"])
        res["vs_reference_pdl"] = vs
        res["vs_reference_pdl_note"] = ("the reference PDL 2.106's own outputs on the same inputs "
                                        "(plain float32 loops for sumover/average/cumusumover; "
                                        "their error, not ours, dominates these figures)")
    return res


def run_family(args, P, torch, stream, hbm):
    """float64 (4096, 2048) Ufunc family on rotating device copies."""
    host = c1_input()
    copies = []
    for _ in range(NCOPIES):
        x = P.pdl(host).to_device()
        x.storage.host = None
        x.storage.fresh = "dev"
        copies.append(x)
    outs = {op: getattr(P, op)(copies[0]) for op in UFUNC_OPS}
    P.sync()

    def one_step(k, ev):
        n = 0
        for j, op in enumerate(UFUNC_OPS):
            x = copies[(k * len(UFUNC_OPS) + j) % NCOPIES]
            if ev is not None:
                ev[j][0].record(stream)
            getattr(P, op)(x, outs[op])
            if ev is not None:
                ev[j][1].record(stream)
            n += P.last_launch_info()["nlaunches"]
        return n

    total, per_op, launches, clocks = timed_steps(torch, stream, args.steps, args.warmup,
                                                  one_step, len(UFUNC_OPS))
    step_bytes = sum(op_bytes(op) for op in UFUNC_OPS)
    ms = total / args.steps
    op_ms = {op: statistics.mean(per_op[j]) for j, op in enumerate(UFUNC_OPS)}
    fx, err = pdl_fixtures(), {}
    if fx is not None:
        for op in UFUNC_OPS:
            got = outs[op].numpy()
            if op == "cumusumover":
                err[op] = errs(got[::32, ::16], fx["c1/cumusumover/sample"])
                err[op]["sample"] = "rows ::32, positions ::16"
            elif f"c1/{op}" in fx.files:
                err[op] = errs(got, fx[f"c1/{op}"])
    return {"workload": FAMILY, "ops": UFUNC_OPS, "error_vs_reference_pdl": err,
            "l2": f"inputs rotate over {NCOPIES} device copies ({NCOPIES * N0 * N1 * 8 >> 20} MiB)",
            "value": step_bytes / (ms * 1e-3) / 1e9, "unit": "GB/s", "ms_per_step": ms,
            "frac_of_hbm": step_bytes / (ms * 1e-3) / 1e9 / hbm,
            "per_op_gbs": {op: op_bytes(op) / (v * 1e-3) / 1e9 for op, v in op_ms.items()},
            "per_op_ms": op_ms, "gpu_launches": launches, "clocks": clocks}


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
            gpu_lead(torch)
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
            diff = np.abs(cn[z][rows].astype(np.float64) - ref)
            diff = np.where(np.isnan(diff), np.inf, diff)  # a NaN result is an error
            err = max(err, float(np.max(diff) / np.max(np.abs(ref))))
        out[name] = {"tflops": flops / (ms * 1e-3) / 1e12, "ms": ms, "kernel": kern,
                     "max_normwise_rel_err": err}
        fx = pdl_fixtures()
        if fx is not None and NB == 16:
            # the reference PDL's float32 matmult: batches 0 and 11, rows (h) ::256
            e = errs(cn[[0, 11]][:, ::256, :], fx["c3m/sample"])
            out[name]["error_vs_reference_pdl"] = {k: v for k, v in e.items() if k != "bit_exact"}
    P.set_matmult_mode(P.MATMULT_BF16X6)
    out["config"] = f"a(t=1024,h=2048) x b(w=2048,t=1024), batch {NB}, float32 N(0,1) seed 4"
    out["speedup_bf16x6_vs_simt"] = out["bf16x6"]["tflops"] / out["simt_fp32"]["tflops"]
    out["tensor_peak_tflops"] = bf16
    out["tensor_peak_kind"] = peak_kind
    return out


# ------------------------------------------------------------- CPU baseline

def gpu_lead(torch):
    """A 1 ms GPU sleep enqueued before a timed call: the call's kernels are
    queued behind it, so the start event does not count the host's planning
    and launch latency (the headline's timed region starts the same way)."""
    torch.cuda._sleep(int(2.0e9 * 0.001))


def time_op(torch, stream, fn, steps, warmup=3):
    """Median device time (ms) of fn() on the library's stream."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        gpu_lead(torch)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def bench_c2(args, P, torch, stream):
    """Config 2: c = sumover(a*b + a), a (256,1,8192), b (256,512,1) ->
    (512,8192), fused in one pass: int32 U{-1000..1000} (seed 2) and float32
    N(0,1) with 2 % BAD in a and in b (seed 3)."""
    out = {}
    nops = 3 * 256 * 512 * 8192
    nbytes = 4 * (256 * 8192 + 256 * 512 + 512 * 8192)
    rng = np.random.default_rng(2)
    a = rng.integers(-1000, 1001, size=(8192, 1, 256)).astype(np.int32)
    b = rng.integers(-1000, 1001, size=(1, 512, 256)).astype(np.int32)
    rng3 = np.random.default_rng(3)
    af = rng3.standard_normal((8192, 1, 256)).astype(np.float32)
    bf = rng3.standard_normal((1, 512, 256)).astype(np.float32)
    bad = np.float32(-3.4028234663852886e38)
    af[rng3.random(af.shape) < 0.02] = bad
    bf[rng3.random(bf.shape) < 0.02] = bad
    variants = {"int32": (a, b, False), "float32_bad": (af, bf, True)}
    for name, (ha, hb, badflag) in variants.items():
        if name not in args.c2_types.split(","):
            continue
        x, y = P.pdl(ha), P.pdl(hb)
        if badflag:
            x.badflag(1)
            y.badflag(1)
        x.to_device()
        y.to_device()
        c = P.sumover_mult_plus(x, y, x)
        P.sync()
        kern = P.last_launch_info()["kernel"]
        ms = time_op(torch, stream, lambda: P.sumover_mult_plus(x, y, x, c), args.mm_steps + 7)
        out[name] = {"ms": ms, "gops": nops / (ms * 1e-3) / 1e9,
                     "gbs": nbytes / (ms * 1e-3) / 1e9, "kernel": kern}
        # the same expression through the generic deferred-expression kernel
        # (one warp per output row, no tile reuse) and eagerly, op by op
        from pdl_gb300.lazy import _run_fused
        e = P.lazy(x) * y + x
        leaves, nodes = e._program()
        ce = _run_fused("sumover", leaves, nodes, None)
        P.sync()
        same = bool(np.array_equal(ce.numpy(), c.numpy())) if name == "int32" else None
        ms_e = time_op(torch, stream, lambda: _run_fused("sumover", leaves, nodes, ce), args.mm_steps + 7)
        ms_g = time_op(torch, stream, lambda: P.sumover(P.plus(P.mult(x, y), x)), 3)
        out[name].update({"expr_generic_ms": ms_e, "eager_chain_ms": ms_g,
                          "expr_generic_equals_tiled": same})
        # output rows (dim 1) ::2048 against the reference PDL and in FP64
        got = c.numpy()[::2048]
        fx = pdl_fixtures()
        if fx is not None:
            out[name]["error_vs_reference_pdl"] = errs(got, fx["c2i/sample" if name == "int32"
                                                             else "c2f/sample"])
        av, bv = ha[::2048, 0, :].astype(np.float64), hb[0].astype(np.float64)   # (4,256), (512,256)
        t = av[:, None, :] * bv[None, :, :] + av[:, None, :]
        if badflag:
            good = (ha[::2048, 0, :] != bad)[:, None, :] & (hb[0] != bad)[None, :, :]
            ref = np.where(good, t, 0.0).sum(-1)
            ref = np.where(good.any(-1), ref, float(bad))
        else:
            ref = t.sum(-1)
        e64 = errs(got, ref)
        out[name]["error_vs_fp64"] = {k: v for k, v in e64.items() if k != "bit_exact"}
    out["config"] = ("sumover(a*b+a): a (256,1,8192), b (256,512,1) -> (512,8192); "
                     "int32 U{-1000..1000} seed 2; float32 N(0,1) seed 3 with 2% BAD")
    out["bound"] = "int32 / fp32 pipe (3 ops per element evaluation, ~120 ops per byte)"
    return out


def c4_inputs():
    """X PDL dims (t=512, h=8192), W (w=256, t=512), bias (w=256): the
    seeded generator shared with the tests."""
    import config_inputs as CI
    d = CI.c4()
    return d["X"], d["W"], d["bias"]


def bench_c4(args, P, torch, stream):
    """Adjoint workload: L = sumover(sumover((matmult(X,W) + bias)**2)) / 8192,
    X float32 dims (512, 8192), W (256, 512), bias (256), N(0, 0.1), seed 6.
    Forward through the ops, backward through the hand-written adjoint calls
    (intermediates recomputed, nothing stored but the inputs and the
    forward's outputs), gradients into preallocated buffers.  Accuracy: FP64
    central finite differences (eps 1e-3) on 64 coordinates (24 of X, 24 of
    W, 16 of bias; the loss change of one coordinate summed from the terms it
    changes), and the hand-derived FP64 gradient everywhere."""
    X, Wm, bias = c4_inputs()
    x, w, b = P.pdl(X).to_device(), P.pdl(Wm).to_device(), P.pdl(bias).to_device()
    Y = P.matmult(x, w)
    Z = P.plus(Y, b)
    S = P.mult(Z, Z)
    s1 = P.sumover(S)
    L = P.sumover(s1)
    gL = P.pdl(np.array(1.0 / 8192, np.float32)).to_device()
    g_s1 = P.sumover_bwd(gL, s1)
    g_S = P.sumover_bwd(g_s1, S)
    gz1, gz2 = P.mult_bwd(g_S, Z, Z)
    g_Z = P.plus(gz1, gz2)
    g_Y, g_b = P.plus_bwd(g_Z, Y, b)
    g_X, g_W = P.matmult_bwd(g_Y, x, w)
    P.sync()

    def fwd():
        P.matmult(x, w, Y)
        P.plus(Y, b, Z)
        P.mult(Z, Z, S)
        P.sumover(S, s1)
        P.sumover(s1, L)

    def bwd():
        P.sumover_bwd(gL, s1, out=g_s1)
        P.sumover_bwd(g_s1, S, out=g_S)
        P.mult_bwd(g_S, Z, Z, out=(gz1, gz2))
        P.plus(gz1, gz2, g_Z)
        P.plus_bwd(g_Z, Y, b, out=(g_Y, g_b))
        P.matmult_bwd(g_Y, x, w, out=(g_X, g_W))

    reps = args.mm_steps + 7
    ms_f = time_op(torch, stream, fwd, reps)
    ms_b = time_op(torch, stream, bwd, reps)
    ms_t = time_op(torch, stream, lambda: (fwd(), bwd()), reps)
    fwd_flop = 2.0 * 512 * 256 * 8192
    bwd_flop = 2 * fwd_flop
    # accuracy against FP64
    gX, gW, gb = g_X.numpy().astype(np.float64), g_W.numpy().astype(np.float64), g_b.numpy().astype(np.float64)
    X64, W64, b64 = X.astype(np.float64), Wm.astype(np.float64), bias.astype(np.float64)
    Z64 = X64 @ W64 + b64                                    # (h, w)
    gZ = 2.0 * Z64 / 8192.0
    ref = {"X": gZ @ W64.T, "W": X64.T @ gZ, "bias": gZ.sum(0)}
    got = {"X": gX, "W": gW, "bias": gb}
    normwise = {k: float(np.max(np.abs(got[k] - ref[k])) / np.max(np.abs(ref[k]))) for k in ref}
    fx = pdl_fixtures()
    vs_pdl = None
    if fx is not None and "c4/gbias" in fx.files:
        # against dL/dX, dL/dW, dL/dbias written out by hand in PDL (float64)
        pdl_g = {"X": (gX[::256], fx["c4/gX/sample"]), "W": (gW[::8], fx["c4/gW/sample"]),
                 "bias": (gb, fx["c4/gbias"])}
        vs_pdl = {k: errs(g, w) for k, (g, w) in pdl_g.items()}
    rng = np.random.default_rng(60)
    eps, fd_err = 1e-3, 0.0

    def dloss(rows_old, rows_new):
        return float(((rows_new * rows_new).sum() - (rows_old * rows_old).sum()) / 8192.0)
    for name, n in [("X", 24), ("W", 24), ("bias", 16)]:
        arr = {"X": X64, "W": W64, "bias": b64}[name]
        for i in rng.choice(arr.size, n, replace=False):
            if name == "X":
                h, t = divmod(int(i), 512)
                old = Z64[h]
                lp, lm = dloss(old, old + eps * W64[t]), dloss(old, old - eps * W64[t])
            elif name == "W":
                t, wv = divmod(int(i), 256)
                old = Z64[:, wv]
                lp, lm = dloss(old, old + eps * X64[:, t]), dloss(old, old - eps * X64[:, t])
            else:
                old = Z64[:, int(i)]
                lp, lm = dloss(old, old + eps), dloss(old, old - eps)
            fd = (lp - lm) / (2 * eps)
            g = float(got[name].reshape(-1)[i])
            fd_err = max(fd_err, abs(g - fd) / max(abs(fd), 1e-4))
    return {"config": "L = sumover(sumover((matmult(X,W)+bias)**2))/8192, X float32 (512,8192), "
                      "W (256,512), bias (256), N(0,0.1) seed 6",
            "fwd_ms": ms_f, "bwd_ms": ms_b, "fwd_bwd_ms": ms_t,
            "fwd_tflops": fwd_flop / (ms_f * 1e-3) / 1e12,
            "bwd_tflops": bwd_flop / (ms_b * 1e-3) / 1e12,
            "max_rel_err_vs_fp64_central_fd_64_coords": fd_err,
            "max_normwise_err_vs_fp64_gradient": normwise,
            "error_vs_gradient_by_hand_in_reference_pdl": vs_pdl,
            "kernels": "k_mm_tc_bf16x6 (matmult and its adjoints), k_biop, k_red_rows, k_unb_*"}


def bench_inner(args, P, torch, stream, hbm):
    """Config 3 inner: float64 a, b dims (4096, 65536), U[-1,1) -> 65536."""
    cols = args.inner_cols
    rng = np.random.default_rng(5)
    a = rng.uniform(-1.0, 1.0, size=(cols, 4096))
    b = rng.uniform(-1.0, 1.0, size=(cols, 4096))
    x, y = P.pdl(a).to_device(), P.pdl(b).to_device()
    a8, b8 = a[::8].copy(), b[::8].copy()
    del a, b
    c = P.inner(x, y)
    P.sync()
    kern = P.last_launch_info()["kernel"]
    ms = time_op(torch, stream, lambda: P.inner(x, y, c), args.mm_steps + 7)
    nbytes = 2 * 4096 * cols * 8 + cols * 8
    gbs = nbytes / (ms * 1e-3) / 1e9
    res = {"config": f"inner, float64 a,b dims (4096,{cols}) U[-1,1) seed 5 -> {cols}",
           "ms": ms, "gbs": gbs, "frac_of_hbm": gbs / hbm, "kernel": kern,
           "gflops": 2 * 4096 * cols / (ms * 1e-3) / 1e9}
    got = c.numpy()[::8]
    fx = pdl_fixtures()
    if fx is not None and cols == 65536:
        res["error_vs_reference_pdl"] = errs(got, fx["c3i/sample"])
        res["error_vs_reference_pdl"]["sample"] = "every 8th output"
    ref = np.array([math.fsum(r) for r in a8 * b8])      # exactly rounded sums of the FP64 products
    res["error_vs_exact_sum"] = {k: v for k, v in errs(got, ref).items() if k != "bit_exact"}
    return res


def bench_expr(args, P, torch, stream, hbm):
    """A deferred expression reduced in one pass, HBM-bound: sumover((a-b)*(a-b))
    over float32 a, b dims (65536, 4096) N(0,1) (seed 8), against the same
    ops run eagerly (two materialised intermediates)."""
    rows = args.expr_rows
    rng = np.random.default_rng(8)
    a = rng.standard_normal((rows, 65536), dtype=np.float32)
    b = rng.standard_normal((rows, 65536), dtype=np.float32)
    x, y = P.pdl(a).to_device(), P.pdl(b).to_device()
    sample = np.arange(0, rows, 64)
    ref = ((a[sample].astype(np.float64) - b[sample]) ** 2).sum(-1)
    del a, b
    d = P.lazy(x) - y
    e = d * d
    c = e.sumover()
    P.sync()
    op = P.last_launch_info()["op"]
    ms = time_op(torch, stream, lambda: e.sumover(c), args.mm_steps + 7)

    def eager():
        t = P.minus(x, y)
        return P.sumover(P.mult(t, t))
    ms_eager = time_op(torch, stream, eager, 3)
    nbytes = 2 * rows * 65536 * 4 + rows * 4
    gbs = nbytes / (ms * 1e-3) / 1e9
    e64 = errs(c.numpy()[sample], ref)
    return {"config": f"sumover((a-b)*(a-b)), float32 a,b dims (65536,{rows}) N(0,1) seed 8 -> {rows}",
            "ms": ms, "gbs": gbs, "frac_of_hbm": gbs / hbm, "op": op,
            "eager_ms": ms_eager, "speedup_vs_eager": ms_eager / ms,
            "error_vs_fp64": {"max_rel_err": e64["max_rel_err"], "normwise_err": e64["normwise_err"],
                              "sample": "every 64th output, FP64 from the float32 inputs"}}


def bench_sort(args, P, torch, stream, hbm):
    """Sort-based reductions: medover and qsorti over float32 dims (100, 65536)
    (65536 rows of 100 values, N(0,1), seed 9: a per-pixel median of a
    100-frame stack); the oracle (the reference's quicksort in C, all host
    threads) on 8192 of the rows."""
    from oracle import oracle as O
    rng = np.random.default_rng(9)
    a = rng.standard_normal((65536, 100), dtype=np.float32)
    x = P.pdl(a).to_device()
    out = {"config": "medover and qsorti, float32 dims (100, 65536) N(0,1) seed 9"}
    nbytes = 65536 * 100 * 4
    for op in ("medover", "qsorti"):
        r = getattr(P, op)(x)
        P.sync()
        ms = time_op(torch, stream, lambda: getattr(P, op)(x), 5)
        out[op] = {"ms": ms, "rows_per_s": 65536 / (ms * 1e-3), "gbs_in": nbytes / (ms * 1e-3) / 1e9,
                   "kernel": "k_sortred_warp"}
        del r
    xs = P.pdl(np.ascontiguousarray(a[:8192]))
    n = os.cpu_count() or 1
    t0 = time.perf_counter()
    want = O.run("medover", [xs], nthreads=n)
    el = time.perf_counter() - t0
    got = P.medover(x).numpy()[:8192]
    want = want[0].numpy().reshape(got.shape)
    out["medover"]["error_vs_oracle"] = errs(got, want)
    out["medover"]["error_vs_oracle"]["sample"] = "the first 8192 rows"
    out["cpu_medover"] = {"rows_per_s": 8192 / el, "cores": n, "kind": "port",
                          "sample": "8192 of the 65536 rows"}
    out["bound"] = ("a warp per row: bitonic network in shared memory (the reference's "
                    "quicksort on the rows whose result could depend on the sort)")
    # longer rows: a block per row (float32 dims (2048, 4096), N(0,1), seed 12)
    al = np.random.default_rng(12).standard_normal((4096, 2048), dtype=np.float32)
    xl = P.pdl(al).to_device()
    r = P.medover(xl)
    P.sync()
    ms = time_op(torch, stream, lambda: P.medover(xl), 5)
    want = O.run("medover", [P.pdl(np.ascontiguousarray(al[:256]))], nthreads=n)[0].numpy()
    out["medover_rows_of_2048"] = {
        "config": "medover, float32 dims (2048, 4096) N(0,1) seed 12: 4096 rows of 2048",
        "ms": ms, "rows_per_s": 4096 / (ms * 1e-3), "gbs_in": al.nbytes / (ms * 1e-3) / 1e9,
        "kernel": "k_sortred_block", "error_vs_oracle": errs(r.numpy()[:256], want)}
    del r, xl
    # one long row: the median of a whole float32 array of 2^22 values (the
    # merge sort), against the oracle's quicksort of the same row on one core
    aw = np.random.default_rng(13).standard_normal(1 << 22, dtype=np.float32)
    xw = P.pdl(aw).to_device()
    for op in ("medover", "qsort"):
        r = getattr(P, op)(xw)
        P.sync()
        ms = time_op(torch, stream, lambda: getattr(P, op)(xw), 5)
        t0 = time.perf_counter()
        want = O.run(op, [P.pdl(aw)])[0].numpy()
        el = time.perf_counter() - t0
        out[f"{op}_one_row_of_2e22"] = {
            "config": "float32 dims (4194304) N(0,1) seed 13: one row",
            "ms": ms, "gbs_in": aw.nbytes / (ms * 1e-3) / 1e9,
            "kernel": "k_lsort_tile + k_lsort_merge + k_lsort_finish",
            "error_vs_oracle": errs(np.atleast_1d(r.numpy()), np.atleast_1d(want)),
            "cpu_port_ms": el * 1e3}
        del r
    del xw
    # vector sorts: 512 planes of 2048 points in 3-D (float64, N(0,1), seed 11)
    v = np.random.default_rng(11).standard_normal((512, 2048, 3))
    xv = P.pdl(v).to_device()
    vbytes = v.nbytes
    for op in ("qsortvec", "qsortveci"):
        r = getattr(P, op)(xv)
        P.sync()
        ms = time_op(torch, stream, lambda: getattr(P, op)(xv), 5)
        want = O.run(op, [P.pdl(np.ascontiguousarray(v[:16]))], nthreads=n)[0].numpy()
        out[op] = {"config": "float64 dims (3, 2048, 512): 512 planes of 2048 3-vectors, N(0,1) seed 11",
                   "ms": ms, "planes_per_s": 512 / (ms * 1e-3), "gbs_in": vbytes / (ms * 1e-3) / 1e9,
                   "kernel": "k_qsortvec_block",
                   "error_vs_oracle": errs(r.numpy()[:16], want)}
        del r
    t0 = time.perf_counter()
    O.run("qsortvec", [P.pdl(np.ascontiguousarray(v[:64]))], nthreads=n)
    out["cpu_qsortvec"] = {"planes_per_s": 64 / (time.perf_counter() - t0), "cores": n,
                           "kind": "port", "sample": "64 of the 512 planes"}
    return out


def bench_fastraw(args, P, torch, stream):
    """FastRaw to device memory: a float32 file of 1 GiB (PDL dims
    (65536, 4096), seeded N(0,1)) written by writefraw to the local temp
    directory, then read straight into device memory by readfraw(device=True)
    (file reads through two pinned staging buffers, the reads overlapping
    the host-to-device copies) and by mapfraw + to_device (the file mapped,
    one copy from the mapping).  The file was just written, so it is read
    from the page cache: these time the host side and the link, not a disk."""
    import tempfile
    rows = 4096
    a = np.random.default_rng(10).standard_normal((rows, 65536), dtype=np.float32)
    nbytes = a.nbytes
    out = {"config": f"float32 PDL dims (65536, {rows}), {nbytes >> 20} MiB, page cache warm"}
    with tempfile.TemporaryDirectory() as td:
        name = os.path.join(td, "c5f")
        P.writefraw(P.pdl(a), name)
        for how, fn in (("readfraw_device", lambda: P.readfraw(name, device=True)),
                        ("mapfraw_to_device", lambda: P.mapfraw(name, ReadOnly=True).to_device())):
            x = fn()
            P.sync()
            ts = []
            for _ in range(3):
                del x
                t0 = time.perf_counter()
                x = fn()
                P.sync()
                ts.append(time.perf_counter() - t0)
            ok = bool(np.array_equal(x.numpy()[::997], a[::997]))
            del x
            out[how] = {"s": statistics.median(ts), "gbs": nbytes / statistics.median(ts) / 1e9,
                        "sampled_rows_equal": ok}
    return out


def cpu_time(arrays, nthreads, budget_s, steps=None):
    """The oracle (the reference's loops in C, with its auto-pthread split
    over the broadcast dims) on the config-5 workload's arrays, every op on
    each; GB/s over the C5 ops.  Runs `steps` steps, or as many as fit in
    budget_s (at least one)."""
    import pdl_gb300 as P
    from oracle import oracle as O
    xs = []
    step_bytes = 0
    for arr in arrays:
        x = P.pdl(np.ascontiguousarray(arr))
        x.badflag(1)
        xs.append(x)
        n, rows = arr.shape[-1], int(np.prod(arr.shape[:-1]))
        step_bytes += sum(op_bytes(op, n, rows, 4, 4) for op in C5_OPS)
    done, t0 = 0, time.perf_counter()
    while True:
        for op in C5_OPS:
            for x in xs:
                O.run(op, [x], nthreads=nthreads)
        done += 1
        el = time.perf_counter() - t0
        if (steps is not None and done >= steps) or (steps is None and el > budget_s):
            break
    return step_bytes * done / el / 1e9, done, el, step_bytes


def cpu_baseline(args, mat, row):
    n = os.cpu_count() or 1
    arrays = [mat] + ([row.reshape(1, -1)] if row is not None else [])
    gbs, steps, el, _ = cpu_time(arrays, n, args.cpu_budget)
    return {"value": gbs, "unit": "GB/s", "cores": n, "kind": "port",
            "sample": f"the whole workload ({'matrix and 2^27 row' if row is not None else 'matrix'}), "
                      f"the 3 ops, {steps} repetitions in {el:.1f} s, auto-pthread split over "
                      f"{n} threads (the reference's; a single row runs on one thread, as in PDL)"}


def run_reference(args, rank, world):
    mat, row = c5_inputs(args.c5_rows)
    arrays = [mat, row.reshape(1, -1)]
    n = os.cpu_count() or 1
    cpu_time(arrays, n, 0.0, steps=max(1, args.warmup))
    ts = []
    for _ in range(args.steps):
        gbs, _, el, sb = cpu_time(arrays, n, 0.0, steps=1)
        ts.append(el)
    value = sb / statistics.mean(ts) / 1e9
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.mean(ts) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded numpy lognormal(0,4), random sign, 1% BAD)",
            "config": {"workload": WORKLOAD, "ops_per_step": C5_OPS,
                       "sample": "the whole workload every step (the matrix and the 2^27 row)"},
            "cpu_baseline": {"value": value, "unit": "GB/s", "cores": n, "kind": "port",
                             "sample": "the whole workload every step; the reference's "
                                       f"auto-pthread split over {n} threads (the 2^27 row, "
                                       "one broadcast iteration, on one thread as in PDL)"},
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
                    help="comma-separated subset of the float64 family (for profiling)")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--c5-rows", type=int, default=C5_ROWS,
                    help="rows of the (65536, rows) matrix (smaller for profiling)")
    ap.add_argument("--c5-ops", default=",".join(C5_OPS))
    ap.add_argument("--no-accuracy", dest="accuracy", action="store_false")
    ap.add_argument("--no-family", dest="family", action="store_false")
    ap.add_argument("--no-secondary", dest="secondary", action="store_false",
                    help="skip the fused sumover(a*b+a) and float64 inner timings")
    ap.add_argument("--inner-cols", type=int, default=65536,
                    help="broadcast length of the float64 inner (smaller for profiling)")
    ap.add_argument("--expr-rows", type=int, default=4096,
                    help="rows of the deferred-expression workload (smaller for profiling)")
    ap.add_argument("--expr-only", action="store_true",
                    help="time only the deferred-expression workload and print its object")
    ap.add_argument("--sort-only", action="store_true",
                    help="time only the sort-based workload and print its object")
    ap.add_argument("--family-only", action="store_true",
                    help="time only the float64 family (--ops) and print its object")
    ap.add_argument("--mm-only", action="store_true",
                    help="time only the float32 matmult workload and print its object")
    ap.add_argument("--inner-only", action="store_true",
                    help="time only the inner leg and print its object")
    ap.add_argument("--c4-only", action="store_true",
                    help="time only the adjoint workload and print its object")
    ap.add_argument("--c2-only", action="store_true",
                    help="time only the fused sumover(a*b+a) workload and print its object")
    ap.add_argument("--c2-types", default="int32,float32_bad",
                    help="comma-separated subset of int32,float32_bad (for profiling)")
    args = ap.parse_args()
    UFUNC_OPS = [o for o in args.ops.split(",") if o]
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, rank, world)))
        return 0
    if (args.expr_only or args.sort_only or args.family_only or args.c2_only or args.c4_only
            or args.mm_only or args.inner_only):
        import torch
        import pdl_gb300 as P
        stream = torch.cuda.current_stream()
        P.set_stream(stream.cuda_stream)
        if args.c2_only or args.c4_only:
            print(json.dumps((bench_c2 if args.c2_only else bench_c4)(args, P, torch, stream)))
            return 0
        if args.mm_only:
            hbm, bf16, kind = peaks()
            print(json.dumps(bench_matmult(args, P, torch, stream, bf16, kind)))
            return 0
        fn = (bench_expr if args.expr_only else bench_sort if args.sort_only
              else bench_inner if args.inner_only else run_family)
        print(json.dumps(fn(args, P, torch, stream, peaks()[0])))
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
