"""Benchmark: weighted model counts/sec on a sliced cubic vertex-cover plan.

Workload: weighted cubic vertex cover, seeded random 3-regular graph, n=220
vertices / 330 edge clauses, cachet weights p ~ U(0.3, 0.7), line-Flow plan
sliced into 2^10 equal-shape slices (frozen in
``tensororder_gb300/plans/wvc220_s10.json.gz`` with the reference's own count).
One step = one complete weighted count (all 1024 slices, compensated FP64 slice
sum).  ``value`` is counts/sec of the chosen (split) form with the plan already
resident on the device; ``e2e`` is the same metric through the plugin's public
call with host inputs (program upload, contraction, result read-back).

With ``--gpus N`` (torchrun, one rank per GPU) one count is split by slice
range: rank r contracts its contiguous block of slices into a compensated
partial, and every step ends with the ranks' 16-byte partials gathered and
combined in rank order -- the design of ``tensororder_gb300/sharding.py``
(strong scaling: the total work per step is one count whatever N is).

``--impl reference`` times the reference algorithm on the host cores instead
(the numpy FP64 restatement in ``oracle/``: the reference's compiled parts are
not available on the GPU machine), on a bounded sample of slices per step: the
line's ``ms_per_step`` is the sample's own time and ``value`` extrapolates the
sample to counts/s.
"""
import argparse
import glob
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


def workload_config(prog, world):
    """The ``config`` of both arms (identical dicts): the workload and its
    work per count, from the plan alone."""
    from tensororder_gb300 import costmodel

    cost = costmodel.executed_cost(prog)
    table = costmodel.join_table(prog)
    return {
        "workload": "weighted cubic vertex cover n=220 (330 clauses), line-Flow, 2^10 slices",
        "slices": prog.num_slices, "joins": prog.num_joins, "max_rank": int(cost["max_rank"]),
        "algorithmic_flop_per_count": float(cost["flops_reference_order"]),
        "executed_flop_per_count": float(cost["flops"]),
        "slice_invariant_joins": sum(1 for j in table if not j.per_slice),
        "l2": "512 MiB buffer zeroed between timed steps (L2 is 129 MB)",
        "parallelism": "slice ranges over %d GPUs" % world if world > 1 else "single GPU",
    }


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


def traffic_records():
    """DRAM traffic recorded from ncu captures: ``traffic-record:`` lines in
    the summaries under ``profiles/``, each naming the join shape, kernel and
    slice count it was captured on."""
    recs = []
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        with open(path) as f:
            for line in f:
                if line.startswith("traffic-record:"):
                    rec = json.loads(line.split(":", 1)[1])
                    rec["source"] = os.path.relpath(path, ROOT)
                    recs.append(rec)
    return recs


_SAMPLE_CODE = r"""
import json, os, sys, time
sys.path.insert(0, sys.argv[1])
import bench
from oracle import contract as oracle
doc, prog = bench.load_workload()
t0 = time.perf_counter(); n = 0
while n < prog.num_slices and (n < int(sys.argv[3]) or time.perf_counter() - t0 < float(sys.argv[2])):
    oracle.contract(prog, n); n += 1
print(json.dumps({"slices": n, "seconds": time.perf_counter() - t0}))
"""


def cpu_sample(threads=None, max_seconds=12.0, min_slices=2):
    """The numpy restatement of the reference's contraction on this host's
    cores over a prefix sample of the slices, in a child process: all BLAS
    threads, or ``threads`` of them (environment set before numpy loads).
    Returns (counts/s extrapolated to the full count, sample description)."""
    env = dict(os.environ)
    if threads is not None:
        for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "BLIS_NUM_THREADS"):
            env[var] = str(threads)
    r = subprocess.run([sys.executable, "-c", _SAMPLE_CODE, ROOT, str(max_seconds), str(min_slices)], env=env,
                       capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError("CPU sample failed: %s" % r.stderr[-2000:])
    out = json.loads(r.stdout.strip().splitlines()[-1])
    per_slice = out["seconds"] / out["slices"]
    return 1.0 / (per_slice * 1024), out


def cpu_baseline():
    """All host cores, plus the single-thread leg."""
    value, s = cpu_sample()
    value1, s1 = cpu_sample(threads=1, max_seconds=10.0)
    return {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "first %d of 1024 slices (%.1f s), numpy FP64 np.tensordot on all host BLAS threads, "
                      "extrapolated to the full count" % (s["slices"], s["seconds"]),
            "single_thread": {"value": value1, "unit": UNIT, "cores": 1,
                              "sample": "first %d of 1024 slices (%.1f s) with BLAS limited to one thread"
                                        % (s1["slices"], s1["seconds"])}}


def batch_line(args, dev):
    """The uneven 512-instance batch (weighted cubic vertex cover n in [30,160]
    and random 3-CNF v in [40,52], each with its own plan and 1..2^8 slices) as
    one CUDA graph per step: counts/s, executed TFLOP/s and the worst error
    against the reference.  Instances with the reference's full count are
    checked on the batch's counts; the others on the slice prefix recorded for
    them, contracted separately (untimed) and compared with the reference's
    count of that prefix."""
    import torch

    from tensororder_gb300 import batch, runtime
    from tensororder_gb300.run_batch import load, reference_errors

    progs, refs, items = load(os.path.join(ROOT, "tensororder_gb300", "plans", "batch512.json.gz"))
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
    full, prefix = reference_errors(progs, items, counts, runtime.MODE_SPLIT, dev.index or 0, stream)
    rel = np.concatenate([full, prefix])
    return {"instances": len(progs), "slices": work["slices"], "ms_per_step": ms,
            "counts_per_s": len(progs) * 1e3 / ms, "executed_tflops": work["executed_flops"] / (ms * 1e-3) / 1e12,
            "max_rel_err_vs_reference": float(rel.max()), "checked": int(rel.size),
            "checked_full_count": int(full.size), "checked_slice_prefix": int(prefix.size),
            "steps": args.batch_steps, "form": "split", "graph": "one CUDA graph per step, 16 internal streams"}


def int_forms_line(prog, dev, steps=3):
    """The unweighted count of the same plan (every variable weight 1) in the
    int forms: the int form (the count modulo 2^64) and the residue form (one
    prime) per count with the plan resident, and the exact ``bigint`` count
    through the plugin (split-form bound, int form, the primes the bound
    needs, Chinese remainder theorem).  Host wall clock after one warm-up
    count; not part of the headline metric."""
    import copy

    import torch

    from tensororder_gb300 import api, exact, runtime

    unweighted = copy.deepcopy(prog)
    for leaf in unweighted.leaves:
        if leaf.kind == "var":
            leaf.w_neg, leaf.w_pos = 1.0, 1.0
    out = {"workload": "the headline plan with every variable weight 1 (its unweighted count)"}
    dp = runtime.DeviceProgram(unweighted, dev.index or 0)
    try:
        dp.set_modulus(exact.MODULI[0])
        words = {}
        for name, mode in (("int64", runtime.MODE_INT64), ("residue", runtime.MODE_MOD)):
            ws = dp.allocate_workspace(mode, unweighted.num_slices, max_fraction=0.3)
            ms = []
            for i in range(1 + steps):
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
                dp.reset()
                dp.run(mode, workspace=ws)
                words[name] = int(dp.result_words(dtype=np.uint64).reshape(-1)[0])
                if i:
                    ms.append((time.perf_counter() - t0) * 1e3)
            out[name + "_ms_per_count"] = float(np.mean(ms))
            del ws
    finally:
        dp.close()
    backend = api.GB300API(device=dev.index or 0)
    backend.add_argument("entry_type", "bigint")
    x = backend.contract_program(unweighted)  # warm-up: lowering, workspaces
    ms = []
    for _ in range(max(1, steps - 1)):
        t0 = time.perf_counter()
        x = backend.contract_program(unweighted)
        ms.append((time.perf_counter() - t0) * 1e3)
    out.update({"bigint_ms_per_count": float(np.mean(ms)), "bigint_bits": int(x).bit_length(),
                "bigint_low_word_equals_int64": int(x) % (1 << 64) == words["int64"],
                "bigint_residue_equals_residue_form": int(x) % exact.MODULI[0] == words["residue"]})
    return out


def run_reference(args, rank, world):
    doc, prog = load_workload()
    if rank != 0:
        return
    from oracle import contract as oracle

    sample = max(1, args.ref_sample)
    S = prog.num_slices
    for w in range(args.warmup):
        oracle.contract(prog, w % S)
    times = []
    for step in range(args.steps):
        t0 = time.perf_counter()
        for s in range(sample):
            oracle.contract(prog, (step * sample + s) % S)
        times.append(time.perf_counter() - t0)
    ms_step = float(np.mean(times)) * 1e3
    value = sample / S / (ms_step * 1e-3)  # counts/s: the sample's share of a count per second
    desc = ("%d of %d slices per step (the sample's own time is ms_per_step; value extrapolates it to whole "
            "counts), numpy FP64 np.tensordot restating the reference's contraction over the same frozen plan, "
            "all host BLAS threads" % (sample, S))
    single, s1 = cpu_sample(threads=1, max_seconds=10.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded 3-regular graph, frozen reference plan)",
        "config": workload_config(prog, world),
        "sample": desc,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": desc,
                         "single_thread": {"value": single, "unit": UNIT, "cores": 1,
                                           "sample": "first %d of 1024 slices (%.1f s) with BLAS limited to one "
                                                     "thread" % (s1["slices"], s1["seconds"])}},
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
    ap.add_argument("--no-int-forms", action="store_true")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    # The CPU baseline runs first, in child processes, before this process
    # touches the GPU.
    cpu = cpu_baseline() if rank == 0 and not args.no_cpu_baseline else None

    import torch
    import torch.distributed as dist

    from tensororder_gb300 import api, runtime, sharding

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
    begin, end = sharding.slice_range(S, rank, world)
    config = workload_config(prog, world)
    flops = config["algorithmic_flop_per_count"]
    flops_exec = config["executed_flop_per_count"]
    ws_split = dp.allocate_workspace(runtime.MODE_SPLIT, S, max_fraction=0.6)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def one(mode, ws):
        """One count: this rank's slices, then (N > 1) the partials combined."""
        dp.reset(stream)
        dp.run(mode, begin, end, workspace=ws, stream=stream)
        if world > 1:
            return float(sharding.combine(sharding.gather_partials(dp.partial(stream))).reshape(-1)[0])
        return None

    def timed(mode, ws, steps, warmup):
        for _ in range(warmup):
            one(mode, ws)
        torch.cuda.synchronize(dev)
        if world > 1:
            dist.barrier()
        ms = []
        val = None
        for _ in range(steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            val = one(mode, ws)
            b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b))
        if val is None:
            val = float(dp.result(stream).reshape(-1)[0])  # the last step's count
        return ms, val

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
        dp.reset(stream)
        dp.run(mode, 0, S, workspace=ws, stream=stream)
        torch.cuda.synchronize(dev)
        t = dp.join_times()
        dp.set_timing(False)
        return t

    jinfo = dp.joins(runtime.MODE_SPLIT)  # (log2 M, log2 N, log2 K, kernel, per slice) per join
    jt_split = per_join(runtime.MODE_SPLIT, dp.allocate_workspace(runtime.MODE_SPLIT, S, 0.6))
    top = int(np.argmax(jt_split))
    mb, nb, kb, kern, per_slice = (int(x) for x in jinfo[top])
    m, n, k = 1 << mb, 1 << nb, 1 << kb
    runs = S if per_slice else 1
    top_flops = 2.0 * m * n * k * runs
    top_bytes = 4.0 * (m * k + k * n + m * n) * runs
    fp64_peak = runtime.probe_peak(0, stream)
    dmma_peak = runtime.probe_peak(2, stream)
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
        # The resource that binds the tensor-core kernel: shared memory.  Every
        # 32-wide K chunk of a 128 x BN tile moves seven chunk-sizes through it:
        # the TMA write, the converters' read and their hi and lo writes, and
        # the MMAs' reads (hi.lo, lo.hi, hi.hi: three operand pairs).
        a, b = (nb, mb) if (mb < 7 and nb > mb) else (mb, nb)  # the kernel tiles 128 rows of the larger
        bn = 128 if b >= 7 else 64
        tiles = max(1, (1 << a) // 128) * max(1, (1 << b) // bn) * runs
        chunks = tiles * ((max(1, k // 8) + 3) // 4)
        smem_bytes = 7.0 * chunks * 4 * 32 * (128 + bn)
        sm_mhz = clocks.summary().get("sm_mhz") or peaks.get("sm_max_mhz") or 2070.0
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        per_clk = smem_bytes / (jt_split[top] * 1e-3) / sms / (sm_mhz * 1e6)
        roof["smem_roofline"] = {
            "bytes_per_launch": smem_bytes, "achieved_bytes_per_clk_per_sm": per_clk,
            "peak_bytes_per_clk_per_sm": 128.0, "frac": per_clk / 128.0, "sm_mhz": sm_mhz, "sms": sms,
            "model": "7 x (128 + BN) x 32 x 4 bytes per K chunk of 32 per tile (TMA write, converter read, "
                     "hi and lo writes, three MMA operand-pair reads); peak = 32 banks x 4 bytes per clock"}
    else:  # memory-bound CUDA-core kernels
        roof = {"bound": "hbm", "achieved": top_bytes / (jt_split[top] * 1e-3) / 1e9,
                "peak": peaks.get("hbm_gbs") or 6800.0, "unit": "GB/s",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks.get("hbm_gbs") else "fallback 6.8 TB/s"}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof.update({"kernel": "join %d (M,N,K)=(%d,%d,%d) x %d slices, %s kernel, split form"
                           % (top, m, n, k, runs, runtime.KERNEL_NAMES[kern]),
                 "share_of_step": float(jt_split[top] / jt_split.sum()),
                 "algorithmic_bytes": top_bytes, "traffic": None,
                 "traffic_source": "no ncu capture recorded for join (%d,%d,%d) on the %s kernel"
                                   % (mb, nb, kb, runtime.KERNEL_NAMES[kern])})
    for rec in traffic_records():
        if tuple(rec["join_mnk"]) == (mb, nb, kb) and rec["kernel_id"] == kern:
            # DRAM bytes of the capture, scaled to the slices of one launch
            # (the traffic grows with the slices processed).
            roof["traffic"] = (rec["dram_read_bytes"] + rec["dram_write_bytes"]) * runs / rec["slices"]
            roof["traffic_source"] = "%s: ncu capture of %s on %d slices, scaled by %d/%d" % (
                rec["source"], rec["kernel"], rec["slices"], runs, rec["slices"])

    # End to end through the public calls: host program in, count out -- the
    # plugin on one GPU; with N ranks each uploads the program, contracts its
    # slice range and the partials are combined (sharding.contract_sharded).
    backend = api.GB300SplitAPI(device=local)

    def e2e_count():
        if world == 1:
            return float(backend.contract_program(prog))
        dpe = runtime.DeviceProgram(prog, local)
        wse = dpe.allocate_workspace(runtime.MODE_SPLIT, max(1, end - begin))
        run = sharding.device_range_runner(dpe, runtime.MODE_SPLIT, wse, stream)
        v = float(sharding.contract_sharded(S, run, rank, world).reshape(-1)[0])
        dpe.close()
        return v

    e2e_ms = []
    for i in range(args.warmup + max(3, args.steps // 2)):
        torch.cuda.synchronize(dev)
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        val = e2e_count()
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_ms.append((t1 - t0) * 1e3)
    if world > 1:
        t = torch.tensor([float(np.mean(e2e_ms))], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = [float(t.item())]
    h2d = int(dp.h2d_bytes)  # leaf parameters (clause/variable leaves are built on the device) + dense leaves
    d2h = 16 * (1 << int(info.root_rank))
    fp64_best = max(fp64_peak, dmma_peak)

    line = {
        "metric": METRIC,
        "value": 1e3 / ms_split,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_split,
        "higher_is_better": True,
        "scaling": "strong",
        "vs_baseline": None,
        "dtype": "f32+pow2-exponent (FP64 compensated slice sum)",
        "data": "synthetic (seeded 3-regular graph, frozen reference plan)",
        "config": config,
        "tflops": flops_exec / (ms_split * 1e-3) / 1e12,
        "tflops_algorithmic": flops / (ms_split * 1e-3) / 1e12,
        "rel_err": abs(split_val - ref) / ref,
        "plain_f64": {"ms_per_count": ms_plain, "counts_per_s": 1e3 / ms_plain,
                      "tflops": flops_exec / (ms_plain * 1e-3) / 1e12, "rel_err": abs(plain_val - ref) / ref},
        "speedup_chosen_vs_plain": ms_plain / ms_split,
        "roofline": roof,
        "step_by_kernel_ms": {kk: {"joins": c, "ms": round(t, 3)} for kk, (c, t) in by_kernel.items()},
        "fp64_roofline": {"achieved_tflops": flops_exec / (ms_plain * 1e-3) / 1e12, "peak_tflops": fp64_best / 1e12,
                          "frac": (flops_exec / (ms_plain * 1e-3)) / fp64_best,
                          "fma_chain_tflops": fp64_peak / 1e12, "dmma_m8n8k4_tflops": dmma_peak / 1e12,
                          "peak_source": "the higher of two togb_probe_peak figures measured in this run: FP64 FMA "
                                         "chains and FP64 mma.sync m8n8k4 (the FP64 tensor pipe)"},
        "clocks": clocks.summary(),
        "e2e": {"value": 1e3 / float(np.mean(e2e_ms)), "unit": UNIT,
                "h2d_bytes_per_step": h2d * world, "d2h_bytes_per_step": d2h * world,
                "path": "GB300SplitAPI.contract_program(host program) -> libtogb C ABI" if world == 1 else
                        "per rank: DeviceProgram(host program) + its slice range, partials combined by "
                        "sharding.contract_sharded"},
        # per count: the fused slice-invariant lists and other slice-invariant joins, then per
        # chunk the slice base, the per-slice joins and the root
        "gpu_launches": launches_per_count * args.steps,
    }
    if not args.no_batch and world == 1:
        line["batch512"] = batch_line(args, dev)
    if not args.no_int_forms and world == 1:
        try:
            line["int_forms"] = int_forms_line(prog, dev)
        except Exception as exc:  # a side figure: it never costs the bench line
            line["int_forms"] = {"error": "%s: %s" % (type(exc).__name__, exc)}
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if world > 1:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
