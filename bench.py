"""Benchmark: SpMV effective GB/s (% of the HBM roofline) on one GB300.

Default workload: powerlaw8m FP32 -- 8,388,608^2 CSR, Zipf(1.8) row lengths on
[1,65,536], 70% of columns within +-4,096 of the diagonal, 30% uniform (about
184M nonzeros, 1.57 GB of algorithmic traffic).  One step = one
y = A*x through a plan of the C ABI (merge-path tile kernel + carry fix-up),
inputs resident in HBM.  The matrix (1.5 GB) is larger than the 129 MB L2, so
no flush is needed between steps.

Algorithmic bytes per SpMV (the roofline numerator):
    nnz*(sizeof(val)+4) + (rows+1)*4 + rows*sizeof(val) + distinct_cols*sizeof(val)

Arms:
  --impl ours (default)   GPU, plus the e2e number through the same C-ABI call
                          with host x / y (H2D + SpMV + D2H in the timed region)
                          and the CPU baseline timed on a bounded sample.
  --impl reference        the reference's CPU CSR loop (oracle port,
                          tests/deep_analysis_runner.cpp:184-190) over the same
                          matrix on all host cores.
Multi-GPU: the path does not shard (one SpMV per matrix); --gpus N runs N
independent replicas, one per rank, and reports the summed throughput.
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

METRIC = "spmv_effective_GBps"
UNIT = "GB/s"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(rows, nnz, distinct, vsize):
    return nnz * (vsize + 4) + (rows + 1) * 4 + rows * vsize + distinct * vsize


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}

        def num(s):
            try:
                return float(s)
            except ValueError:
                return None

        sm = [num(r[1]) for r in self.rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in self.rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in self.rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_matrix(mx, W, name, dtype, seed=0, scale_rows=0):
    spec = W.scaled(name, scale_rows, seed) if scale_rows else W.spec(name, seed)
    t = time.time()
    rp, ci, v = mx.generate(spec, dtype=dtype)
    x = mx.gen_vector(spec.numCols, W.x_seed(seed), dtype=dtype)
    return spec, rp, ci, v, x, time.time() - t


def cpu_reference_arm(args):
    """The reference's CPU CSR loop on all host threads (oracle port)."""
    import muxi_spmv_gb300 as mx
    from muxi_spmv_gb300 import workloads as W
    import oracle

    ws, rank, _ = dist_env()
    if rank != 0:
        return
    dtype = np.float32 if args.dtype == "f32" else np.float64
    spec, rp, ci, v, x, _ = make_matrix(mx, W, args.workload, dtype, scale_rows=args.scale_rows)
    vs = np.dtype(dtype).itemsize
    distinct = oracle.distinct_columns(ci, spec.numCols)
    nbytes = algorithmic_bytes(spec.numRows, len(ci), distinct, vs)
    threads = os.cpu_count() or 1
    y = np.empty(spec.numRows, dtype)
    for _ in range(args.warmup):
        oracle.cpu_spmv(rp, ci, v, x, threads=threads, out=y)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle.cpu_spmv(rp, ci, v, x, threads=threads, out=y)
        times.append(time.perf_counter() - t)
    tot = sum(times)
    val = nbytes * args.steps / tot / 1e9
    line = {"metric": METRIC, "value": round(val, 3), "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(tot / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": args.workload, "rows": spec.numRows, "nnz": int(len(ci)),
                       "algorithmic_bytes": int(nbytes), "parallelism": "replicas"},
            "cpu_baseline": {"value": round(val, 3), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"full {args.workload} matrix, one SpMV pass per step, row-parallel "
                                       f"reference loop (deep_analysis_runner.cpp:184-190) on {threads} threads"},
            "e2e": {"value": round(val, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def gpu_arm(args):
    import torch

    import muxi_spmv_gb300 as mx
    from muxi_spmv_gb300 import workloads as W
    import oracle

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dtype = np.float32 if args.dtype == "f32" else np.float64
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    vs = np.dtype(dtype).itemsize

    spec, rp, ci, v, xh, gen_s = make_matrix(mx, W, args.workload, dtype, seed=0, scale_rows=args.scale_rows)
    A = mx.CSRMatrix(rp, ci, v, spec.numCols).copyToDevice(dev)
    stream = torch.cuda.Stream(device=dev)
    h = mx.spmv_create_handle()
    h.set_stream(stream)
    var = None
    if args.variant:
        k, b, t, i, w = (int(z) for z in args.variant.split(","))
        var = mx.make_variant(k, b, t, i, w)
    plan = mx.Plan(h, A, var)
    distinct = mx.count_distinct_columns(A, stream)
    nbytes = algorithmic_bytes(A.numRows, A.nnz, distinct, vs)
    x = torch.from_numpy(xh).to(dev)
    y = torch.empty(A.numRows, dtype=tdt, device=dev)

    # Parity of the benchmarked matrix (full size) against the FP64 oracle.
    with torch.cuda.stream(stream):
        plan.exec(x, y)
    stream.synchronize()
    plan.device_error()  # raises if a bounded pipeline wait gave up
    y_ref, absum = oracle.spmv_ref(rp, ci, v, xh)
    ratio = oracle.row_errors(y.cpu().numpy(), y_ref, absum, 1e-5 if dtype == np.float32 else 1e-13)
    parity = {"rows_checked": int(A.numRows), "max_err_over_bound": float(ratio.max()),
              "rows_out_of_bound": int((ratio > 1).sum())}
    if parity["rows_out_of_bound"]:
        print(f"PARITY FAILURE: {parity}", file=sys.stderr)

    # ---- device-resident timing ------------------------------------------
    for _ in range(args.warmup):
        plan.exec(x, y)
    stream.synchronize()
    if ws > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    plan.profile(True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(args.steps):
        plan.exec(x, y)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    step_ms = e0.elapsed_time(e1) / args.steps
    kern_ms_total, kern_launches = plan.profile_read()
    plan.profile(False)

    # ---- end to end: host x in, host y out, through the same C-ABI call ----
    x_pin = torch.from_numpy(xh).pin_memory()
    y_pin = torch.empty(A.numRows, dtype=tdt).pin_memory()
    with torch.cuda.stream(stream):
        for _ in range(max(1, args.warmup)):
            x.copy_(x_pin, non_blocking=True)
            plan.exec(x, y)
            y_pin.copy_(y, non_blocking=True)
    stream.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        f0.record(stream)
        for _ in range(args.steps):
            x.copy_(x_pin, non_blocking=True)
            plan.exec(x, y)
            y_pin.copy_(y, non_blocking=True)
        f1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = f0.elapsed_time(f1) / args.steps
    plan.device_error()
    clocks.stop()

    if ws > 1:
        t = torch.tensor([step_ms, e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms, e2e_ms = t.tolist()
        dist.barrier()

    peak, peak_kind = peaks()
    kern_ms = kern_ms_total / max(kern_launches, 1)
    achieved = nbytes / (kern_ms * 1e-3) / 1e9
    value = ws * nbytes / (step_ms * 1e-3) / 1e9
    e2e_val = ws * nbytes / (e2e_ms * 1e-3) / 1e9
    pv = plan.variant.as_dict()
    launches_per_step = 2 if pv["kernel"] == mx.KERNEL_MERGE else 1

    traffic = None
    tf = ROOT / "profiles" / f"traffic_{args.workload}_{args.dtype}.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get("dram_bytes_per_launch")
        except Exception:
            traffic = None

    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(step_ms, 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded generators)",
            "config": {"workload": args.workload, "rows": A.numRows, "cols": A.numCols, "nnz": A.nnz,
                       "distinct_cols": distinct, "algorithmic_bytes": int(nbytes), "variant": pv,
                       "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas{ws}",
                       "gflops": round(2 * A.nnz / (step_ms * 1e-3) / 1e9, 2), "generate_s": round(gen_s, 2)},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                         "kernel": "merge_tile_kernel" if launches_per_step == 2 else "csr_rows_kernel",
                         "kernel_ms": round(kern_ms, 5), "traffic": traffic},
            "e2e": {"value": round(e2e_val, 3), "unit": UNIT, "h2d_bytes_per_step": int(A.numCols * vs),
                    "d2h_bytes_per_step": int(A.numRows * vs), "ms_per_step": round(e2e_ms, 5),
                    "call": "spmv_plan_exec_f32 with host x/y copied in the timed region"},
            "gpu_launches": args.steps * launches_per_step * 2,
            "clocks": clocks.summary(), "parity": parity}

    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        yc = np.empty(A.numRows, dtype)
        oracle.cpu_spmv(rp, ci, v, xh, threads=threads, out=yc)  # warm
        reps, t = 0, time.perf_counter()
        while reps < 3 or (time.perf_counter() - t < 5.0 and reps < 50):
            oracle.cpu_spmv(rp, ci, v, xh, threads=threads, out=yc)
            reps += 1
        cpu_s = (time.perf_counter() - t) / reps
        t = time.perf_counter()
        oracle.cpu_spmv(rp, ci, v, xh, threads=1, out=yc)
        ser_s = time.perf_counter() - t
        line["cpu_baseline"] = {"value": round(nbytes / cpu_s / 1e9, 3), "unit": UNIT, "cores": threads,
                                "kind": "port",
                                "sample": f"full matrix, {reps} row-parallel passes of the reference CPU loop",
                                "serial_value": round(nbytes / ser_s / 1e9, 3), "serial_cores": 1}
    if rank == 0:
        print(json.dumps(line), flush=True)
    plan.destroy()
    h.destroy()
    if ws > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="powerlaw8m")
    ap.add_argument("--dtype", default="f32", choices=["f32", "f64"])
    ap.add_argument("--variant", default="", help="kernel,block,tpr,ipt,vec (spmv_variant_t)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--scale-rows", type=int, default=0, help="same law on this many rows (profiling cases)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        cpu_reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
