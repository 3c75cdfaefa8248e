"""Benchmark: weighted model counts/sec on a sliced cubic vertex-cover plan.

Workload: weighted cubic vertex cover, seeded random 3-regular graph, n=220
vertices / 330 edge clauses, cachet weights p ~ U(0.3, 0.7), line-Flow plan
sliced into 2^10 equal-shape slices (frozen in
``tensororder_gb300/plans/wvc220_s10.json.gz`` with the reference's own count).
One step = one complete weighted count (all 1024 slices, compensated FP64 slice
sum).  ``value`` is counts/sec of the chosen (split) form with the plan already
resident on the device; ``e2e`` is the same metric through the plugin's public
call with host inputs (program upload, contraction, result read-back).

``--impl reference`` times the reference algorithm on the host cores instead
(the numpy FP64 restatement in ``oracle/``: the reference's compiled parts are
not available on this machine), on a bounded sample of slices per step.
"""
import argparse
import gzip
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "wvc220_s10"
METRIC = "weighted counts/sec (chosen split form, all 1024 slices per count)"
UNIT = "counts/s"


def load_workload(name=WORKLOAD):
    from tensororder_gb300.program import Program

    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", name + ".json.gz"), "rt") as f:
        doc = json.load(f)
    return doc, Program.from_dict(doc["program"])


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def cpu_baseline(prog, max_seconds=12.0, min_slices=2):
    """The numpy restatement of the reference's contraction on this host's
    cores, on a prefix sample of the slices (bounded by ``max_seconds``)."""
    from oracle import contract as oracle

    t0 = time.perf_counter()
    n = 0
    total = 0.0
    while n < prog.num_slices and (n < min_slices or time.perf_counter() - t0 < max_seconds):
        arr, _ = oracle.contract(prog, n)
        total += float(arr[()])
        n += 1
    dt = time.perf_counter() - t0
    per_slice = dt / n
    return {"value": 1.0 / (per_slice * prog.num_slices), "unit": UNIT, "cores": os.cpu_count(),
            "kind": "port",
            "sample": "first %d of %d slices (%.1f s), numpy FP64 np.tensordot on all host BLAS threads, "
                      "extrapolated to the full count" % (n, prog.num_slices, dt)}


def batch_line(args, dev):
    """The uneven 512-instance batch (weighted cubic vertex cover n in [30,160]
    and random 3-CNF v in [40,52], each with its own plan and 1..2^8 slices) as
    one CUDA graph per step: counts/s, executed TFLOP/s and the worst error
    against the reference's counts recorded for 252 of the instances."""
    import torch

    from tensororder_gb300 import batch, runtime
    from tensororder_gb300.run_batch import load

    progs, refs, _ = load(os.path.join(ROOT, "tensororder_gb300", "plans", "batch512.json.gz"))
    ex = batch.BatchExecutor(progs, runtime.MODE_SPLIT, device=dev.index or 0, nstreams=16)
    stream = torch.cuda.current_stream(dev)
    ex.run(stream)  # warm-up (graph upload)
    torch.cuda.synchronize(dev)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(max(1, args.batch_steps)):
        ex.run(stream)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b) / max(1, args.batch_steps)
    counts = ex.counts(stream)
    work = ex.work()
    ex.close()
    have = ~np.isnan(refs)
    rel = np.abs(counts[have] - refs[have]) / np.abs(refs[have])
    return {"instances": len(progs), "slices": work["slices"], "ms_per_step": ms,
            "counts_per_s": len(progs) * 1e3 / ms, "executed_tflops": work["executed_flops"] / (ms * 1e-3) / 1e12,
            "max_rel_err_vs_reference": float(rel.max()), "checked": int(have.sum()), "steps": args.batch_steps,
            "form": "split", "graph": "one CUDA graph per step, 16 internal streams"}


def run_reference(args, rank, world):
    doc, prog = load_workload()
    if rank != 0:
        return
    from oracle import contract as oracle

    sample = max(1, args.ref_sample)
    for _ in range(args.warmup):
        oracle.contract(prog, 0)
    times = []
    for step in range(args.steps):
        t0 = time.perf_counter()
        for s in range(sample):
            oracle.contract(prog, (step * sample + s) % prog.num_slices)
        times.append((time.perf_counter() - t0) / sample)
    per_slice = float(np.mean(times))
    value = 1.0 / (per_slice * prog.num_slices)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_slice * prog.num_slices * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "slices": prog.num_slices, "joins": prog.num_joins,
                   "per_step_sample_slices": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "sample": "%d slices per step of %d, numpy FP64 (the reference's np.tensordot "
                                   "contraction restated over the same frozen plan), all host BLAS threads"
                                   % (sample, prog.num_slices)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--ref-sample", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-steps", type=int, default=2)
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import torch.distributed as dist

    from tensororder_gb300 import api, runtime

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    doc, prog = load_workload()
    ref = doc["reference"]["float64"]
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)

    dp = runtime.DeviceProgram(prog, local)
    info = dp.info
    S = prog.num_slices
    # Algorithmic FLOP per count as the reference performs it: every join of
    # every slice.  Executed FLOP: slice-invariant joins run once per count.
    flops = (info.flops_per_slice + info.flops_once) * S
    flops_exec = info.flops_per_slice * S + info.flops_once
    ws_split = dp.allocate_workspace(runtime.MODE_SPLIT, S, max_fraction=0.6)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def one(mode, ws):
        dp.reset(stream)
        dp.run(mode, 0, S, workspace=ws, stream=stream)

    def timed(mode, ws, steps, warmup):
        for _ in range(warmup):
            one(mode, ws)
        torch.cuda.synchronize(dev)
        ms = []
        for _ in range(steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            one(mode, ws)
            b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b))
        val = float(dp.result(stream).reshape(-1)[0])  # the last step's count
        return ms, val

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clocks:
        split_ms, split_val = timed(runtime.MODE_SPLIT, ws_split, args.steps, args.warmup)
    torch.cuda.synchronize(dev)
    launches_per_count = dp.launch_count(runtime.MODE_SPLIT)  # as the timed steps queued them
    t_split = float(np.sum(split_ms)) / 1e3
    if world > 1:
        t = torch.tensor([t_split], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_split = float(t.item())
    ms_split = t_split * 1e3 / args.steps

    # Plain FP64 form on the same plan (the 10x comparison).
    ws_plain = dp.allocate_workspace(runtime.MODE_F64, S, max_fraction=0.6)
    plain_ms, plain_val = timed(runtime.MODE_F64, ws_plain, args.plain_steps, 1)
    ms_plain = float(np.mean(plain_ms))

    # Per-join device times of one instrumented pass of each form (CUDA events
    # between launches on the launching stream).
    def per_join(mode, ws):
        dp.set_timing(True)
        one(mode, ws)
        torch.cuda.synchronize(dev)
        t = dp.join_times()
        dp.set_timing(False)
        return t

    jinfo = dp.joins(runtime.MODE_SPLIT)  # (log2 M, log2 N, log2 K, kernel, per slice) per join
    jt_split = per_join(runtime.MODE_SPLIT, dp.allocate_workspace(runtime.MODE_SPLIT, S, 0.6))
    jt_plain = per_join(runtime.MODE_F64, dp.allocate_workspace(runtime.MODE_F64, S, 0.6))
    top = int(np.argmax(jt_split))
    mb, nb, kb, kern, per_slice = (int(x) for x in jinfo[top])
    m, n, k = 1 << mb, 1 << nb, 1 << kb
    runs = S if per_slice else 1
    top_flops = 2.0 * m * n * k * runs
    top_bytes = 4.0 * (m * k + k * n + m * n) * runs
    fp32_peak = runtime.probe_peak(1, stream)
    fp64_peak = runtime.probe_peak(0, stream)
    tf32_peak = runtime.probe_peak(3, stream)
    peaks = measured_peaks()
    by_kernel = {}
    for j in range(len(jt_split)):
        name = runtime.KERNEL_NAMES[int(jinfo[j][3])]
        c, t = by_kernel.get(name, (0, 0.0))
        by_kernel[name] = (c + 1, t + float(jt_split[j]))
    if kern == 3:  # tensor cores: 3 TF32 MMAs per product
        roof = {"bound": "tensor", "achieved": top_flops / (jt_split[top] * 1e-3) / 1e12,
                "peak": tf32_peak / 3 / 1e12, "unit": "TFLOP/s",
                "peak_source": "tcgen05 kind::tf32 probe measured in this run (%.0f TFLOP/s) / 3 MMAs per "
                               "3xTF32 product" % (tf32_peak / 1e12),
                "tensor_pipe_tflops": 3 * top_flops / (jt_split[top] * 1e-3) / 1e12,
                "bf16_measured_tflops": peaks.get("bf16_tflops")}
    else:  # memory-bound CUDA-core kernels
        roof = {"bound": "hbm", "achieved": top_bytes / (jt_split[top] * 1e-3) / 1e9,
                "peak": peaks.get("hbm_gbs") or 6800.0, "unit": "GB/s",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks.get("hbm_gbs") else "fallback 6.8 TB/s"}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof.update({"kernel": "join %d (M,N,K)=(%d,%d,%d) x %d slices, %s kernel, split form"
                           % (top, m, n, k, runs, runtime.KERNEL_NAMES[kern]),
                 "share_of_step": float(jt_split[top] / jt_split.sum()),
                 "algorithmic_bytes": top_bytes, "traffic": None})
    if (mb, nb, kb, kern) == (8, 11, 9, 3):
        # DRAM read + write of this join in an ncu capture (--set full) of its
        # first 32 slices, 151.1 + 39.4 MB, scaled to the slices of one launch.
        roof["traffic"] = (151.11168e6 + 39.404544e6) * runs / 32
        roof["traffic_source"] = "ncu capture of 32 slices scaled by %d/32" % runs

    # End to end through the plugin's public call: host program in, count out.
    backend = api.GB300SplitAPI(device=local)
    e2e_ms = []
    for i in range(args.warmup + max(3, args.steps // 2)):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        val = float(backend.contract_program(prog))
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_ms.append((t1 - t0) * 1e3)
    h2d = int(dp.h2d_bytes)  # leaf parameters (clause/variable leaves are built on the device) + dense leaves
    d2h = 16 * (1 << int(info.root_rank))

    line = {
        "metric": METRIC,
        "value": world * 1e3 / ms_split,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_split,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+pow2-exponent (FP64 compensated slice sum)",
        "data": "synthetic (seeded 3-regular graph, frozen reference plan)",
        "config": {
            "workload": "weighted cubic vertex cover n=220 (330 clauses), line-Flow, 2^10 slices",
            "slices": S, "joins": prog.num_joins, "max_rank": int(info.max_rank),
            "algorithmic_flop_per_count": flops,
            "executed_flop_per_count": flops_exec,
            "slice_invariant_joins": int(info.num_joins_once),
            "l2": "512 MiB buffer zeroed between timed steps (L2 is 129 MB)",
            "parallelism": "replicas" if world > 1 else "single GPU",
        },
        "tflops": flops_exec / (ms_split * 1e-3) / 1e12,
        "tflops_algorithmic": flops / (ms_split * 1e-3) / 1e12,
        "rel_err": abs(split_val - ref) / ref,
        "plain_f64": {"ms_per_count": ms_plain, "counts_per_s": 1e3 / ms_plain,
                      "tflops": flops_exec / (ms_plain * 1e-3) / 1e12, "rel_err": abs(plain_val - ref) / ref},
        "speedup_chosen_vs_plain": ms_plain / ms_split,
        "roofline": roof,
        "step_by_kernel_ms": {kk: {"joins": c, "ms": round(t, 3)} for kk, (c, t) in by_kernel.items()},
        "fp64_roofline": {"achieved_tflops": flops_exec / (ms_plain * 1e-3) / 1e12, "peak_tflops": fp64_peak / 1e12,
                          "frac": (flops_exec / (ms_plain * 1e-3)) / fp64_peak,
                          "peak_source": "togb_probe_peak FP64 FMA chain, measured in this run"},
        "clocks": clocks.summary(),
        "e2e": {"value": 1e3 / float(np.mean(e2e_ms)), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "path": "GB300SplitAPI.contract_program(host program) -> libtogb C ABI"},
        # per count: the fused slice-invariant lists and other slice-invariant joins, then per
        # chunk the slice base, the per-slice joins and the root
        "gpu_launches": launches_per_count * args.steps,
    }
    if not args.no_batch:
        line["batch512"] = batch_line(args, dev)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(prog)
    if world > 1:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
