"""Benchmark: SpMV effective GB/s (% of the HBM roofline) on one GB300.

Default workload: powerlaw8m FP32 -- 8,388,608^2 CSR, Zipf(1.8) row lengths on
[1,65,536], 70% of columns within +-4,096 of the diagonal, 30% uniform (about
184M nonzeros, 1.57 GB of algorithmic traffic).  One step = one
y = A*x through a plan of the C ABI (the default AUTO variant: CSR5 tiles of
256 nonzeros with gathers in nonzero order + carry fix-up), inputs resident in
HBM.  --workload uneven1024 runs the batched uneven SpMV/SpMM instead.  The matrix (1.5 GB) is larger than the 129 MB L2, so
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


def max_over_ranks(values, ws, device):
    """Max of each value over the ranks (replicas: the job takes as long as
    its slowest rank).  One all_reduce on `device` (NCCL on GPUs, gloo on CPU)."""
    if ws <= 1:
        return list(values)
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def replica_throughput(ws, units_per_rank, ms):
    """Whole-job rate: every rank processed `units_per_rank` in at most `ms`."""
    return ws * units_per_rank / (ms * 1e-3)


def make_matrix(mx, W, name, dtype, seed=0, scale_rows=0):
    spec = W.scaled(name, scale_rows, seed) if scale_rows else W.spec(name, seed)
    t = time.time()
    rp, ci, v = mx.generate(spec, dtype=dtype)
    x = mx.gen_vector(spec.numCols, W.x_seed(seed), dtype=dtype)
    return spec, rp, ci, v, x, time.time() - t


def workload_config(workload, rows, cols, nnz, distinct, nbytes, ws):
    """The `config` of both arms: what the workload is, nothing about how it
    is computed (the GPU arm puts its plan under "plan")."""
    return {"workload": workload, "rows": int(rows), "cols": int(cols), "nnz": int(nnz),
            "distinct_cols": int(distinct), "algorithmic_bytes": int(nbytes),
            "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas{ws}"}


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
            "scaling": "weak", "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded generators)",
            "impl": "reference",
            "config": workload_config(args.workload, spec.numRows, spec.numCols, int(len(ci)), distinct, nbytes,
                                      args.gpus),
            "cpu_baseline": {"value": round(val, 3), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"full {args.workload} matrix, one SpMV pass per step: the reference's CPU "
                                       f"CSR loop (deep_analysis_runner.cpp:184-190) restated in oracle/oracle.c, "
                                       f"row-parallel on {threads} threads; the restatement is pinned bit-exact to "
                                       f"the reference loop compiled from its sources (tests/test_oracle_pins.py)"},
            "e2e": {"value": round(val, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


SUB_WORKLOADS = (("poisson16k", "f32"), ("powerlaw8m", "f64"), ("powerlaw8m_c1024", "f32"),
                 ("stencil2d_4096", "f32"), ("stencil3d_256", "f32"))


def time_plan(torch, plan, x, y, stream, dev, steps, warmup):
    """(ms per step, ms of the main kernel per launch): CUDA events on the
    launching stream; the kernel alone from the plan's own event pair."""
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            plan.exec(x, y)
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    with torch.cuda.stream(stream):
        for _ in range(steps):
            plan.exec(x, y)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    step_ms = e0.elapsed_time(e1) / steps
    plan.profile(True)
    with torch.cuda.stream(stream):
        for _ in range(steps):
            plan.exec(x, y)
    km, kl = plan.profile_read()
    plan.profile(False)
    return step_ms, km / max(kl, 1)


def l2_resident_record(torch, plan, x, y, stream, dev, nbytes, l2_bytes):
    """Matrices that fit in L2 (the 16K Poisson case): SpMVs replayed from a
    CUDA graph, warm (matrix and x in L2) and with L2 flushed before each
    SpMV (a buffer twice the L2 written, its own time subtracted).  None when
    the matrix and vectors take more than half the L2."""
    if nbytes * 2 >= l2_bytes:
        return None
    reps, inner = 10, 20
    flush = torch.empty(2 * l2_bytes // 4, dtype=torch.float32, device=dev)

    def graph_ms(body):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            for _ in range(inner):
                body()
        g.replay()
        torch.cuda.synchronize(dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            g.replay()
        b.record(stream)
        torch.cuda.synchronize(dev)
        return a.elapsed_time(b) / (reps * inner)

    with torch.cuda.stream(stream):
        warm = graph_ms(lambda: plan.exec(x, y))
        both = graph_ms(lambda: (flush.fill_(1.0), plan.exec(x, y)))
        fl = graph_ms(lambda: flush.fill_(1.0))
    del flush
    return {"graph_warm": {"value": round(nbytes / (warm * 1e-3) / 1e9, 3), "us_per_spmv": round(warm * 1e3, 3)},
            "graph_l2_flushed": {"value": round(nbytes / (max(both - fl, 1e-6) * 1e-3) / 1e9, 3),
                                 "us_per_spmv": round((both - fl) * 1e3, 3)},
            "note": f"matrix + vectors {int(nbytes)} B fit the {l2_bytes} B L2; {reps}x{inner} SpMVs per figure "
                    "from one CUDA graph; flushed = (flush + SpMV) - flush, flush = writing twice the L2"}


def sub_record(args, mx, W, oracle, h, stream, dev, name, dt, peak):
    """One compact record of another benchmark configuration: full-size
    matrix, the AUTO plan, full-size parity against the FP64 oracle, step
    and kernel GB/s with the clocks sampled during the timed region."""
    import torch
    dtype = np.float32 if dt == "f32" else np.float64
    vs = np.dtype(dtype).itemsize
    spec, rp, ci, v, xh, gen_s = make_matrix(mx, W, name, dtype, seed=0)
    A = mx.CSRMatrix(rp, ci, v, spec.numCols).copyToDevice(dev)
    plan = mx.Plan(h, A)
    distinct = mx.count_distinct_columns(A, stream)
    nbytes = algorithmic_bytes(A.numRows, A.nnz, distinct, vs)
    x = torch.from_numpy(xh).to(dev)
    y = torch.empty(A.numRows, dtype=x.dtype, device=dev)
    with torch.cuda.stream(stream):
        plan.exec(x, y)
    stream.synchronize()
    plan.device_error()
    y_ref, absum = oracle.spmv_ref(rp, ci, v, xh)
    r = oracle.row_errors(y.cpu().numpy(), y_ref, absum, 1e-5 if dtype == np.float32 else 1e-13)
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    time.sleep(0.3)
    step_ms, kern_ms = time_plan(torch, plan, x, y, stream, dev, args.steps, args.warmup)
    clocks.stop()
    pv = plan.variant.as_dict()
    rec = {"workload": name, "dtype": dt, "rows": A.numRows, "nnz": A.nnz, "algorithmic_bytes": int(nbytes),
           "variant": pv, "ms_per_step": round(step_ms, 5), "value": round(nbytes / (step_ms * 1e-3) / 1e9, 3),
           "kernel_ms": round(kern_ms, 5), "kernel_GBps": round(nbytes / (kern_ms * 1e-3) / 1e9, 2),
           "frac": round(nbytes / (kern_ms * 1e-3) / 1e9 / peak, 4),
           "parity": {"rows_checked": int(A.numRows), "max_err_over_bound": float(r.max()),
                      "rows_out_of_bound": int((r > 1).sum())},
           "clocks": clocks.summary(), "generate_s": round(gen_s, 2),
           "l2": ("inputs larger than L2 (no flush)" if nbytes * 2 >= int(h.l2CacheBytes) else
                  "fits in L2: value and kernel figures warm; l2_resident.graph_l2_flushed has L2 flushed "
                  "before each SpMV")}
    l2res = l2_resident_record(torch, plan, x, y, stream, dev, nbytes, int(h.l2CacheBytes))
    if l2res is not None:
        rec["l2_resident"] = l2res
    if rec["parity"]["rows_out_of_bound"]:
        print(f"PARITY FAILURE {name} {dt}: {rec['parity']}", file=sys.stderr)
    plan.destroy()
    del A, x, y
    torch.cuda.empty_cache()
    return rec


def selector_record(args, mx, h, A, x, y, stream, dev):
    """The learned kernel pick against the exhaustive autotune on one matrix:
    regret of the pick's time and the ratio of the two selections' costs."""
    import torch
    from muxi_spmv_gb300 import selector as S
    model = S.MLP.load(S.DEFAULT_MODEL)
    space = S.variant_space()
    torch.cuda.synchronize(dev)
    S.select(h, A, S.SELECT_LEARNED, model)  # warm: feature buffers, model upload
    torch.cuda.synchronize(dev)
    t = time.perf_counter()
    reps = 5
    for _ in range(reps):
        learned, li = S.select(h, A, S.SELECT_LEARNED, model)
    torch.cuda.synchronize(dev)
    learned_s = (time.perf_counter() - t) / reps
    t = time.perf_counter()
    fb, fi = S.select(h, A, S.SELECT_LEARNED_FALLBACK, model)
    torch.cuda.synchronize(dev)
    fallback_s = time.perf_counter() - t
    t = time.perf_counter()
    best, bi = S.select(h, A, S.SELECT_AUTOTUNE)
    torch.cuda.synchronize(dev)
    autotune_s = time.perf_counter() - t
    times = {}
    for tag, var in (("learned", learned), ("fallback", fb), ("autotune", best)):
        p = mx.Plan(h, A, var)
        step_ms, _ = time_plan(torch, p, x, y, stream, dev, args.steps, args.warmup)
        times[tag] = step_ms
        p.destroy()
    model.destroy()
    return {"matrix": args.workload, "learned_pick": S.variant_name(space[li]) if li >= 0 else str(learned),
            "fallback_pick": S.variant_name(space[fi]) if fi >= 0 else str(fb),
            "autotune_pick": S.variant_name(space[bi]) if bi >= 0 else str(best),
            "learned_ms": round(times["learned"], 5), "fallback_ms": round(times["fallback"], 5),
            "autotune_ms": round(times["autotune"], 5),
            "regret": round(times["learned"] / times["autotune"] - 1.0, 4),
            "fallback_regret": round(times["fallback"] / times["autotune"] - 1.0, 4),
            "selection_ms": {"learned": round(learned_s * 1e3, 3), "fallback": round(fallback_s * 1e3, 3),
                             "autotune": round(autotune_s * 1e3, 3)},
            "cost_ratio": round(autotune_s / max(learned_s, 1e-9), 1),
            "fallback_cost_ratio": round(autotune_s / max(fallback_s, 1e-9), 1),
            "note": "selection = spmv_select (features + MLP forward + rank), the same with the variants "
                    "predicted within 12% timed, at most four (the mode of the benchmark's AUTO plans), and "
                    "spmv_select(AUTOTUNE) (every applicable variant timed as a plan); regrets from the picks' "
                    "plans timed back to back with CUDA events"}


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
    model = None
    if args.select in ("learned", "learned_fallback") and not args.variant:
        from muxi_spmv_gb300 import selector as S
        model = S.MLP.load(S.DEFAULT_MODEL)
        # AUTO plans take the learned pick; with the fallback, the variants
        # predicted within 12% of it (at most four) are timed at plan creation and the fastest kept
        S.set_selector(h, model, S.SELECT_LEARNED_FALLBACK if args.select == "learned_fallback" else S.SELECT_LEARNED)
    perm = None
    if args.colperm != "none":
        # Column reorder on the GPU (reorderColumns / "RCM" / frequency orders),
        # columns re-sorted within rows; x is permuted to match, y is unchanged.
        kind = {"com": mx.COLPERM_CENTER_OF_MASS, "minrow": mx.COLPERM_MIN_ROW,
                "freq": mx.COLPERM_FREQUENCY}[args.colperm]
        with torch.cuda.stream(stream):
            perm, _ = mx.column_perm(A, kind, stream)
            A.d_colIdx[:A.nnz].copy_(mx.apply_column_perm(A, perm, stream))
            mx.sort_columns_within_rows(A, stream)
        stream.synchronize()
    plan = mx.Plan(h, A, var)
    distinct = mx.count_distinct_columns(A, stream)
    nbytes = algorithmic_bytes(A.numRows, A.nnz, distinct, vs)
    x0 = torch.from_numpy(xh).to(dev)
    x = mx.permute_x(perm, x0, stream) if perm is not None else x0
    stream.synchronize()
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
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(args.steps):
        plan.exec(x, y)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    step_ms = e0.elapsed_time(e1) / args.steps
    # The main kernel alone: the plan records an event pair around it (a
    # separate pass, since an event between the tile kernel and its fix-up
    # keeps the fix-up from launching behind the tile kernel's last wave).
    plan.profile(True)
    for _ in range(args.steps):
        plan.exec(x, y)
    kern_ms_total, kern_launches = plan.profile_read()
    plan.profile(False)

    # ---- end to end: host x in, host y out, through the same C-ABI call ----
    x_pin = torch.from_numpy(xh).pin_memory()
    y_pin = torch.empty(A.numRows, dtype=tdt).pin_memory()
    def e2e_step():
        if perm is None:
            x.copy_(x_pin, non_blocking=True)
        else:  # host x arrives in the original column order
            x0.copy_(x_pin, non_blocking=True)
            mx.check(mx.lib().spmv_permute_x_f32(x.numel(), perm.data_ptr(), x0.data_ptr(), x.data_ptr(),
                                                 stream.cuda_stream) if vs == 4 else
                     mx.lib().spmv_permute_x_f64(x.numel(), perm.data_ptr(), x0.data_ptr(), x.data_ptr(),
                                                 stream.cuda_stream), "permute_x")
        plan.exec(x, y)
        y_pin.copy_(y, non_blocking=True)

    with torch.cuda.stream(stream):
        for _ in range(max(1, args.warmup)):
            e2e_step()
    stream.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        f0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        f1.record(stream)
    torch.cuda.synchronize(dev)
    serial_ms = f0.elapsed_time(f1) / args.steps
    plan.device_error()

    # ---- end to end through the host pipeline (spmv_pipeline_*): each
    # request copies its own x in and its y out; copies overlap the SpMV of
    # the same request (row slices) and of the neighbouring requests.
    pipe_info, pipe_parity = None, None
    e2e_ms = serial_ms
    if perm is None and not args.no_pipeline:
        pipe = mx.Pipeline(h, A, plan.variant, slices=args.slices, depth=args.depth)
        pipe_info = pipe.info()
        xs = [x_pin, torch.from_numpy(mx.gen_vector(A.numCols, 77, dtype=dtype)).pin_memory()]
        ys = [torch.empty(A.numRows, dtype=tdt).pin_memory() for _ in range(2)]
        for i in range(max(1, args.warmup)):
            pipe.submit(xs[i % 2], ys[i % 2])
        pipe.wait()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        pipe.order_after(stream)
        for i in range(args.steps):  # the last request takes xs[0], the x of the parity check
            j = (args.steps - 1 - i) % 2
            pipe.submit(xs[j], ys[j])
        pipe.join(stream)
        g1.record(stream)
        torch.cuda.synchronize(dev)
        pipe.wait()
        e2e_ms = g0.elapsed_time(g1) / args.steps
        r = oracle.row_errors(ys[0].numpy(), y_ref, absum, 1e-5 if dtype == np.float32 else 1e-13)
        pipe_parity = {"rows_checked": int(A.numRows), "max_err_over_bound": float(r.max()),
                       "rows_out_of_bound": int((r > 1).sum())}
        if pipe_parity["rows_out_of_bound"]:
            print(f"PIPELINE PARITY FAILURE: {pipe_parity}", file=sys.stderr)
        pipe.destroy()
    # ---- matrices that fit in L2 (the 16K Poisson case): graph replays
    l2res = l2_resident_record(torch, plan, x, y, stream, dev, nbytes, int(h.l2CacheBytes))

    # ---- the vendor library on the same matrix and x: cuSPARSE SpMV through
    # torch.sparse (context only; nothing of ours on this path).
    vendor = None
    if not args.no_vendor and perm is None:
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            Acsr = torch.sparse_csr_tensor(A.d_rowPtr, A.d_colIdx[:A.nnz], A.d_values[:A.nnz],
                                           size=(A.numRows, A.numCols), check_invariants=False)
            with torch.cuda.stream(stream):
                yv = torch.mv(Acsr, x)
                for _ in range(args.warmup):
                    torch.mv(Acsr, x)
                h0 = torch.cuda.Event(enable_timing=True)
                h1 = torch.cuda.Event(enable_timing=True)
                h0.record(stream)
                for _ in range(args.steps):
                    torch.mv(Acsr, x)
                h1.record(stream)
            torch.cuda.synchronize(dev)
        v_ms = h0.elapsed_time(h1) / args.steps
        r = oracle.row_errors(yv.cpu().numpy(), y_ref, absum, 1e-5 if dtype == np.float32 else 1e-13)
        vendor = {"library": "cuSPARSE SpMV via torch.sparse_csr_tensor / torch.mv (torch " + torch.__version__ + ")",
                  "value": round(nbytes / (v_ms * 1e-3) / 1e9, 3), "unit": UNIT, "ms_per_step": round(v_ms, 5),
                  "rows_out_of_bound": int((r > 1).sum())}
        del Acsr
    clocks.stop()

    step_ms, e2e_ms, serial_ms = max_over_ranks([step_ms, e2e_ms, serial_ms], ws, dev)
    if ws > 1:
        dist.barrier()

    peak, peak_kind = peaks()
    kern_ms = kern_ms_total / max(kern_launches, 1)
    achieved = nbytes / (kern_ms * 1e-3) / 1e9
    value = replica_throughput(ws, nbytes, step_ms) / 1e9
    e2e_val = replica_throughput(ws, nbytes, e2e_ms) / 1e9
    serial_val = replica_throughput(ws, nbytes, serial_ms) / 1e9
    pv = plan.variant.as_dict()
    csr5_name = ("csr5_tile_kernel" if pv["vectorWidth"] < mx.CSR5_ORDERED else
                 "csr5_ordered_range_kernel" if pv["threadsPerRow"] > 0 else "csr5_ordered_kernel")
    kern_names = {mx.KERNEL_MERGE: "merge_vec_kernel", mx.KERNEL_CSR5: csr5_name,
                  mx.KERNEL_BAND: "csr5_window_kernel", mx.KERNEL_STREAM: "csr5_stream_kernel",
                  mx.KERNEL_ELL: "ell_kernel", mx.KERNEL_SCALAR: "csr_rows_kernel", mx.KERNEL_VECTOR: "csr_rows_kernel"}
    # merge-path and the CSR5-tiled plans launch the tile kernel and a carry fix-up
    launches_per_step = 2 if pv["kernel"] in (mx.KERNEL_MERGE, mx.KERNEL_CSR5, mx.KERNEL_BAND,
                                              mx.KERNEL_STREAM) else 1

    traffic = None
    tf = ROOT / "profiles" / f"traffic_{args.workload}_{args.dtype}.json"
    if tf.exists() and perm is None and not args.scale_rows:
        try:  # a capture of this workload's dominant kernel, for the variant it was taken with
            rec = json.loads(tf.read_text())
            if list(rec.get("variant", [])) == [pv[k] for k in ("kernel", "blockSize", "threadsPerRow",
                                                                 "itemsPerThread", "vectorWidth")]:
                traffic = rec.get("dram_bytes_per_launch")
        except Exception:
            traffic = None

    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(step_ms, 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded generators)",
            "config": workload_config(args.workload + (f"+colperm_{args.colperm}" if perm is not None else ""),
                                      A.numRows, A.numCols, A.nnz, distinct, nbytes, ws),
            "plan": {"variant": pv, "select": "explicit variant" if args.variant else args.select,
                     "gflops": round(2 * A.nnz / (step_ms * 1e-3) / 1e9, 2), "generate_s": round(gen_s, 2)},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                         "kernel": kern_names.get(pv["kernel"], str(pv["kernel"])),
                         "kernel_ms": round(kern_ms, 5), "traffic": traffic},
            "e2e": {"value": round(e2e_val, 3), "unit": UNIT, "h2d_bytes_per_step": int(A.numCols * vs),
                    "d2h_bytes_per_step": int(A.numRows * vs), "ms_per_step": round(e2e_ms, 5),
                    "call": ("spmv_pipeline_submit: pinned host x in, pinned host y out, copies overlapped "
                             f"({pipe_info['slices']} row slices, {pipe_info['depth']} requests in flight)"
                             if pipe_info else "spmv_plan_exec with host x/y copied in the timed region"),
                    "serial": {"value": round(serial_val, 3), "ms_per_step": round(serial_ms, 5),
                               "call": "H2D(x), spmv_plan_exec, D2H(y) in order on one stream"},
                    "pipeline_parity": pipe_parity},
            "gpu_launches": args.steps * launches_per_step * 3 +
                            (args.steps * pipe_info["launches_per_request"] if pipe_info else 0),
            "clocks": clocks.summary(), "parity": parity, "vendor_library": vendor, "l2_resident": l2res}

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
                                "sample": f"full matrix, {reps} row-parallel passes of the reference's CPU CSR loop "
                                          "(deep_analysis_runner.cpp:184-190) restated in oracle/oracle.c, which is "
                                          "pinned bit-exact to that loop compiled from the reference's sources "
                                          "(tests/test_oracle_pins.py)",
                                "serial_value": round(nbytes / ser_s / 1e9, 3), "serial_cores": 1}
    if rank == 0 and not args.no_subrecords and not args.scale_rows and perm is None:
        # the other configurations, each through its own AUTO plan, and the
        # learned selector on this matrix (outside the headline's timed region)
        if dtype == np.float32:
            line["selector"] = selector_record(args, mx, h, A, x, y, stream, dev)
        plan.destroy()
        plan = None
        del A, x, y, x0
        torch.cuda.empty_cache()
        line["subrecords"] = [sub_record(args, mx, W, oracle, h, stream, dev, name, dt, peak)
                              for name, dt in SUB_WORKLOADS if (name, dt) != (args.workload, args.dtype)]
        line["subrecords"].append(batch_subrecord(args, mx, oracle, stream, dev, peak, peak_kind))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if plan is not None:
        plan.destroy()
    h.destroy()
    if ws > 1:
        dist.destroy_process_group()


def batch_subrecord(args, mx, oracle, stream, dev, peak, peak_kind):
    """The uneven batch at k=1 (1,024 matrices) as one compact record: the
    persistent launch from a CUDA graph against the two per-matrix loops,
    on a handle of its own (default AUTO plans in the loop, as a user of
    the reference's entry points would make them)."""
    import torch
    from muxi_spmv_gb300 import batch as B
    from muxi_spmv_gb300 import selector as S
    h = mx.spmv_create_handle()
    h.set_stream(stream)
    t0 = time.time()
    mats = [S.gen_device(s.spec) for s in B.uneven_specs(args.batch_count, seed=0)]
    torch.cuda.synchronize(dev)
    gen_s = time.time() - t0
    distinct = [mx.count_distinct_columns(A, stream) for A in mats]
    ctx = dict(mx=mx, B=B, oracle=oracle, h=h, stream=stream, dev=dev, mats=mats, distinct=distinct, rank=0, ws=1,
               local=dev.index or 0, peak=peak, peak_kind=peak_kind, gen_s=gen_s,
               sumR=sum(A.numRows for A in mats), sumC=sum(A.numCols for A in mats), sumN=sum(A.nnz for A in mats))
    rec = batch_k_line(args, ctx, "1", compact=True)
    del mats, ctx
    torch.cuda.empty_cache()
    h.destroy()
    return rec


def batch_k_line(args, ctx, kspec, compact=False):
    """One k of the uneven batch: the JSON line of that k (see batched_arm).
    compact: the persistent graph and the two per-matrix loops only (no
    e2e, no CPU sample), for the record inside the default benchmark line."""
    import torch
    mx, B, oracle, h, stream, dev = (ctx[k] for k in ("mx", "B", "oracle", "h", "stream", "dev"))
    mats, distinct, rank, ws, local = (ctx[k] for k in ("mats", "distinct", "rank", "ws", "local"))
    peak, peak_kind, gen_s, sumR, sumC, sumN = (ctx[k] for k in ("peak", "peak_kind", "gen_s", "sumR", "sumC",
                                                                   "sumN"))
    L = mx.lib()

    def aligned_slices(sizes):
        offs, o = [], 0
        for n in sizes:
            offs.append(o)
            o += (n + 3) // 4 * 4
        return offs, max(o, 4)

    # "mixed": each matrix draws its own k from {1, 2, 4, 8, 16} (seeded);
    # the batch runs as a group of single-k batches in one graph
    mixed = kspec == "mixed"
    if mixed:
        kk = [int(z) for z in np.random.default_rng(4242 + rank).choice([1, 2, 4, 8, 16], len(mats))]
        k = "mixed"
    else:
        k = int(kspec)
        kk = [k] * len(mats)
    xo, xn = aligned_slices([A.numCols * ki for A, ki in zip(mats, kk)])
    yo, yn = aligned_slices([A.numRows * ki for A, ki in zip(mats, kk)])
    Xd = torch.empty(xn, dtype=torch.float32, device=dev)
    Yd = torch.empty(yn, dtype=torch.float32, device=dev)
    mx.check(L.spmv_gen_device_vector_f32(xn, 1000 + (0 if mixed else k), -1.0, 1.0, Xd.data_ptr(), None),
             "gen x")
    xs = [Xd[o:o + A.numCols * ki] for o, A, ki in zip(xo, mats, kk)]
    ys = [Yd[o:o + max(A.numRows * ki, 1)] for o, A, ki in zip(yo, mats, kk)]
    # launch shape picked by the batch autotuner on this batch (per k group)
    if mixed:
        best_v, tune_ms = {}, {}
        for kg in sorted(set(kk)):
            sel_ = [i for i, ki in enumerate(kk) if ki == kg]
            bv, tm = B.autotune_batch(h, [mats[i] for i in sel_], kg, [xs[i] for i in sel_],
                                      [ys[i] for i in sel_], repeats=3, stream=stream)
            best_v[kg] = bv
            tune_ms.update({(kg,) + key: t for key, t in tm.items()})
        plan = B.BatchGroupPlan(h, mats, kk, best_v)
        info = {"tiles": None, "warps": None, "groups": plan.info()["batches"]}
    else:
        best_v, tune_ms = B.autotune_batch(h, mats, k, xs, ys, repeats=3, stream=stream)
        plan = B.BatchPlan(h, mats, k, best_v)
        info = plan.info()
    plan.set_vectors(xs, ys)
    plan.exec(1.0, 0.0, B.BATCH_PERSISTENT_GRAPH)
    stream.synchronize()

    # parity on sampled matrices (all k columns) against the FP64 oracle
    worst, checked = 0.0, 0
    for i in np.linspace(0, len(mats) - 1, args.parity_samples).astype(int):
        A = mats[i]
        rp = A.d_rowPtr.cpu().numpy()
        ci = A.d_colIdx[:A.nnz].cpu().numpy()
        v = A.d_values[:A.nnz].cpu().numpy()
        ki = kk[i]
        X = xs[i].cpu().numpy().reshape(A.numCols, ki)
        Y = ys[i][:A.numRows * ki].cpu().numpy().reshape(A.numRows, ki)
        for j in range(ki):
            yr, absum = oracle.spmv_ref(rp, ci, v, np.ascontiguousarray(X[:, j]))
            worst = max(worst, float(oracle.row_errors(Y[:, j], yr, absum, 1e-5).max()))
            checked += A.numRows
    if worst > 1.0:
        print(f"PARITY FAILURE k={k}: {worst}", file=sys.stderr)

    nbytes = sum(A.nnz * 8 + (A.numRows + 1) * 4 + ki * A.numRows * 4 + ki * d * 4
                 for A, d, ki in zip(mats, distinct, kk))
    sumNK = sum(A.nnz * ki for A, ki in zip(mats, kk))
    times = {}
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    modes = (("persistent_graph", B.BATCH_PERSISTENT_GRAPH, args.steps),
             ("persistent", B.BATCH_PERSISTENT, args.steps),
             ("loop", B.BATCH_LOOP, max(3, args.steps // 4)),
             ("loop_graph", B.BATCH_LOOP_GRAPH, max(3, args.steps // 4)))
    for name, mode, steps in modes[:1] if compact else modes:
        for _ in range(args.warmup):
            plan.exec(1.0, 0.0, mode)
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            plan.exec(1.0, 0.0, mode)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        times[name] = e0.elapsed_time(e1) / steps

    # the plain per-matrix loop a reference user writes: one single-matrix
    # plan per matrix (default AUTO variant), one SpMV per right-hand side
    plans = [mx.Plan(h, A) for A in mats]
    xcols = [xs[i].view(A.numCols, kk[i]).t().contiguous() for i, A in enumerate(mats)]
    ycols = [torch.empty(kk[i], max(A.numRows, 1), dtype=torch.float32, device=dev) for i, A in enumerate(mats)]
    plain_steps = max(2, args.steps // 8)

    def plain_once():
        for p_, xc, yc in zip(plans, xcols, ycols):
            for j in range(xc.shape[0]):
                p_.exec(xc[j], yc[j])
    plain_once()
    stream.synchronize()
    for i in np.linspace(0, len(mats) - 1, 4).astype(int):  # same product as the batch
        A = mats[i]
        ref = ys[i][:A.numRows * kk[i]].view(A.numRows, kk[i]).t()
        assert torch.allclose(ycols[i][:, :A.numRows], ref, rtol=1e-4, atol=1e-4), "plain loop mismatch"
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(plain_steps):
        plain_once()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    times["plain_loop"] = e0.elapsed_time(e1) / plain_steps
    for p_ in plans:
        p_.destroy()
    del plans

    # the same loop through the reference's own entry point: spmv_csr<T>
    # per matrix and right-hand side (stateless: tiles found every call)
    opts = mx.spmv_default_opts(stream)

    def stateless_once():
        for A, xc, yc in zip(mats, xcols, ycols):
            for j in range(xc.shape[0]):
                mx.spmv_csr(A, xc[j], yc[j], 1.0, 0.0, opts)
    stateless_once()
    stream.synchronize()
    e0.record(stream)
    for _ in range(plain_steps):
        stateless_once()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    times["spmv_csr_loop"] = e0.elapsed_time(e1) / plain_steps
    del xcols, ycols

    if compact:
        clocks.stop()
        ms = max_over_ranks([times["persistent_graph"]], ws, dev)[0]
        plan.destroy()
        del Xd, Yd, xs, ys
        torch.cuda.empty_cache()
        return {"workload": f"uneven{len(mats)}", "k": k, "matrices": len(mats), "rows": sumR, "nnz": sumN,
                "algorithmic_bytes": int(nbytes), "variant": best_v, "ms_per_step": round(ms, 5),
                "value": round(ws * 1e3 / ms, 3), "unit": "batch/s",
                "kernel_GBps": round(nbytes / (ms * 1e-3) / 1e9, 2),
                "frac": round(nbytes / (ms * 1e-3) / 1e9 / peak, 4),
                "ms": {n: round(t, 4) for n, t in times.items()},
                "speedup_vs_plain_loop": round(times["plain_loop"] / ms, 3),
                "speedup_vs_spmv_csr_loop": round(times["spmv_csr_loop"] / ms, 3),
                "note": "persistent launch replayed from a CUDA graph against a loop of single-matrix plans "
                        "(plain_loop) and a loop of stateless spmv_csr_f32 calls (spmv_csr_loop)",
                "parity": {"matrices_checked": int(args.parity_samples), "rows_checked": checked,
                           "max_err_over_bound": worst},
                "clocks": clocks.summary(), "generate_s": round(gen_s, 2)}

    # end to end: pinned host X in, Y out, persistent graph in between
    Xh = torch.empty(xn, dtype=torch.float32).pin_memory()
    Yh = torch.empty(yn, dtype=torch.float32).pin_memory()
    Xh.copy_(Xd.cpu())
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            Xd.copy_(Xh, non_blocking=True)
            plan.exec(1.0, 0.0, B.BATCH_PERSISTENT_GRAPH)
            Yh.copy_(Yd, non_blocking=True)
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            Xd.copy_(Xh, non_blocking=True)
            plan.exec(1.0, 0.0, B.BATCH_PERSISTENT_GRAPH)
            Yh.copy_(Yd, non_blocking=True)
        f1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = f0.elapsed_time(f1) / args.steps
    clocks.stop()
    times["persistent_graph"], e2e_ms = max_over_ranks([times["persistent_graph"], e2e_ms], ws, dev)

    ms = times["persistent_graph"]
    achieved = nbytes / (ms * 1e-3) / 1e9
    line = {"metric": "batched_spmm_batches_per_s", "value": round(ws * 1e3 / ms, 3), "unit": "batch/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded device generators)",
            "config": {"workload": f"uneven{args.batch_count}", "k": k,
                       "k_counts": {str(z): kk.count(z) for z in sorted(set(kk))} if mixed else None,
                       "matrices": len(mats), "rows": sumR,
                       "cols": sumC, "nnz": sumN, "algorithmic_bytes": int(nbytes), "tiles": info["tiles"],
                       "warps": info["warps"], "l2": "inputs larger than L2 (no flush)",
                       "parallelism": f"replicas{ws}", "generate_s": round(gen_s, 2),
                       "gflops": round(2 * sumNK / (ms * 1e-3) / 1e9, 2),
                       "ms": {n: round(t, 4) for n, t in times.items()},
                       "variant": {str(z): v for z, v in best_v.items()} if mixed else best_v,
                       "autotune_ms": {",".join(map(str, key)): round(t, 4) for key, t in tune_ms.items()},
                       "speedup_vs_plain_loop": round(times["plain_loop"] / ms, 3),
                       "speedup_vs_spmv_csr_loop": round(times["spmv_csr_loop"] / ms, 3),
                       "spmv_csr_loop": "per matrix and right-hand side: one spmv_csr_f32 call (the reference's "
                                        "spmv_csr<T>, stateless: CSR5 tiles found per call, 3 launches)",
                       "plain_loop": "per matrix: one single-matrix plan (default AUTO variant), one "
                                     "spmv_plan_exec_f32 per right-hand side, 2 launches each",
                       "speedup_vs_loop": round(times["loop"] / ms, 3),
                       "speedup_vs_loop_graph": round(times["loop_graph"] / ms, 3)},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                         "kernel": ("batch_tile_kernel<k> + batch_fixup_kernel<k> per k group (one graph)"
                                    if mixed else f"batch_tile_kernel<{k}> + batch_fixup_kernel<{k}> (graph)"),
                         "traffic": None},
            "e2e": {"value": round(ws * 1e3 / e2e_ms, 3), "unit": "batch/s", "h2d_bytes_per_step": int(xn * 4),
                    "d2h_bytes_per_step": int(yn * 4), "ms_per_step": round(e2e_ms, 5),
                    "call": ("spmv_batch_group_exec_f32" if mixed else "spmv_batch_exec_f32") +
                            " (persistent graph) with pinned X/Y copies"},
            "gpu_launches": 2 * args.steps * (info["groups"] if mixed else 1),
            "clocks": clocks.summary(),
            "parity": {"matrices_checked": int(args.parity_samples), "rows_checked": checked,
                       "max_err_over_bound": worst}}
    if rank == 0 and not args.no_cpu_baseline:
        # bounded sample: the reference CPU loop over 64 matrices, k passes each
        threads = os.cpu_count() or 1
        idx = np.linspace(0, len(mats) - 1, 64).astype(int)
        host = []
        for i in idx:
            A = mats[i]
            host.append((A.d_rowPtr.cpu().numpy(), A.d_colIdx[:A.nnz].cpu().numpy(),
                         A.d_values[:A.nnz].cpu().numpy(), xs[i].cpu().numpy().reshape(A.numCols, kk[i])))
        nn = sum(int(rp[-1]) * X.shape[1] for rp, _, _, X in host)  # nonzero-columns
        t = time.perf_counter()
        for rp, ci, v, X in host:
            for j in range(X.shape[1]):
                oracle.cpu_spmv(rp, ci, v, np.ascontiguousarray(X[:, j]), threads=threads)
        cpu_s = (time.perf_counter() - t) * sumNK / max(nn, 1)
        line["cpu_baseline"] = {"value": round(1.0 / cpu_s, 4), "unit": "batch/s", "cores": threads,
                                "kind": "port",
                                "sample": f"64 of {len(mats)} matrices ({nn} nonzero-columns), reference CPU "
                                          f"loop per column, scaled to the batch's {sumNK} nonzero-columns"}
    plan.destroy()
    del Xd, Yd, xs, ys, Xh, Yh
    torch.cuda.empty_cache()
    return line


def batched_arm(args):
    """Uneven batch: 1,024 CSR matrices (rows log-uniform [1,024, 262,144],
    mean row length U[2,64], Poisson or Zipf(2.0) lengths), k right-hand
    sides.  One JSON line per k: batches/s of the persistent launch replayed
    from a CUDA graph, against the per-matrix loop (plain launches and graph).
    X blocks of all matrices live in one device buffer (16-byte aligned
    slices), so the e2e number moves them with one pinned copy each way."""
    import ctypes as C

    import torch

    import muxi_spmv_gb300 as mx
    from muxi_spmv_gb300 import batch as B
    from muxi_spmv_gb300 import selector as S
    import oracle

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    h = mx.spmv_create_handle()
    h.set_stream(stream)
    t0 = time.time()
    specs = B.uneven_specs(args.batch_count, seed=rank)
    mats = [S.gen_device(s.spec) for s in specs]
    torch.cuda.synchronize()
    gen_s = time.time() - t0
    distinct = [mx.count_distinct_columns(A, stream) for A in mats]
    sumN = sum(A.nnz for A in mats)
    sumR = sum(A.numRows for A in mats)
    sumC = sum(A.numCols for A in mats)
    peak, peak_kind = peaks()
    ctx = dict(mx=mx, B=B, oracle=oracle, h=h, stream=stream, dev=dev, mats=mats, distinct=distinct,
               rank=rank, ws=ws, local=local, peak=peak, peak_kind=peak_kind, gen_s=gen_s, sumR=sumR, sumC=sumC,
               sumN=sumN)
    for kspec in args.k.split(","):
        line = batch_k_line(args, ctx, kspec)
        if rank == 0:
            print(json.dumps(line), flush=True)
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
    ap.add_argument("--no-pipeline", action="store_true", help="e2e through one stream, copies not overlapped")
    ap.add_argument("--no-vendor", action="store_true", help="skip the cuSPARSE comparison")
    ap.add_argument("--no-subrecords", action="store_true",
                    help="skip the other configurations and the selector record (profiling runs)")
    ap.add_argument("--select", default="learned_fallback", choices=["default", "learned", "learned_fallback"],
                    help="AUTO plan: the fixed default variant, the learned selector's pick, or that pick with the "
                         "variants predicted within 12%% of it (at most four) timed at plan creation")
    ap.add_argument("--slices", type=int, default=1, help="host pipeline row slices")
    ap.add_argument("--depth", type=int, default=2, help="host pipeline requests in flight")
    ap.add_argument("--scale-rows", type=int, default=0, help="same law on this many rows (profiling cases)")
    ap.add_argument("--colperm", default="none", choices=["none", "com", "minrow", "freq"],
                    help="reorder columns first (centre of mass, the reference's min-row 'RCM', frequency)")
    ap.add_argument("--k", default="1,2,4,8,16,mixed",
                    help="right-hand sides (uneven batch workload); 'mixed': each matrix draws its own k")
    ap.add_argument("--batch-count", type=int, default=1024, help="matrices (uneven batch workload)")
    ap.add_argument("--parity-samples", type=int, default=8, help="matrices checked (uneven batch workload)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    batched = args.workload.startswith("uneven")
    if args.impl == "reference":
        if batched:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched multi-matrix path"}))
        else:
            cpu_reference_arm(args)
    elif batched:
        batched_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
