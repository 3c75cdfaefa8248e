"""Contract an uneven batch of frozen plans on the GPU and report throughput.

    python -m tensororder_gb300.run_batch BATCH [--mode split|f64] [--steps K]
                                                [--warmup W] [--streams S]
                                                [--tune N] [--limit L]

``BATCH`` is a ``togb.batch/1`` file (``tensororder_gb300/plans/batch512.json.gz``).
All instances (or the first ``L``) are built into one ``togb_batch`` CUDA
graph; one step contracts every instance's full count.  ``--tune N`` first
autotunes the join kernels on the first N instances.  Prints one JSON line:
counts/s, executed TFLOP/s, the worst relative error against the reference's
numpy counts recorded in the batch file, and the autotuner's effect.
"""
from __future__ import annotations

import argparse
import gzip
import json
import sys
import time

import numpy as np

from . import batch, runtime
from .program import Program


def load(path, limit=None):
    with gzip.open(path, "rt") as f:
        doc = json.load(f)
    items = doc["instances"][:limit] if limit else doc["instances"]
    progs = [Program.from_dict(it["program"]) for it in items]
    refs = np.array([np.nan if it["reference_float64"] is None else it["reference_float64"] for it in items])
    return progs, refs, items


def reference_errors(progs, items, counts, mode=runtime.MODE_SPLIT, device=0, stream=None, max_prefix_flops=None):
    """Relative errors of a batch against the reference's counts recorded in
    the batch file: ``counts[i]`` (the batch's full count) for instances with
    the reference's full count, and for the others a separate contraction of
    the recorded slice prefix (``reference_prefix``: the first P slices in
    ``itertools.product`` order, the reference's ``num_slice_limit``,
    ``base_api.py:23-24``).  Instances whose prefix work exceeds
    ``max_prefix_flops`` are skipped.  Returns ``(full, prefix)`` arrays of
    relative errors."""
    full, prefix = [], []
    for i, it in enumerate(items):
        if it["reference_float64"] is not None:
            full.append(abs(counts[i] - it["reference_float64"]) / abs(it["reference_float64"]))
            continue
        pre = it.get("reference_prefix")
        if not pre:
            continue
        P = int(pre["slices"])
        if max_prefix_flops is not None and it["executed_flops"] * P / (1 << it["slice_groups"]) > max_prefix_flops:
            continue
        dp = runtime.DeviceProgram(progs[i], device)
        dp.reset(stream)
        dp.run(mode, 0, P, workspace=dp.allocate_workspace(mode, P), stream=stream)
        got = float(dp.result(stream).reshape(-1)[0])
        dp.close()
        prefix.append(abs(got - pre["float64"]) / abs(pre["float64"]))
    return np.array(full), np.array(prefix)


def time_steps(ex, steps, warmup, stream):
    import torch

    for _ in range(warmup):
        ex.run(stream)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        ex.run(stream)
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b) / steps


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("batch")
    ap.add_argument("--mode", choices=["split", "f64"], default="split")
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--streams", type=int, default=16)
    ap.add_argument("--tune", type=int, default=0)
    ap.add_argument("--limit", type=int, default=None)
    args = ap.parse_args(argv)

    import torch

    mode = runtime.MODE_SPLIT if args.mode == "split" else runtime.MODE_F64
    progs, refs, items = load(args.batch, args.limit)
    stream = torch.cuda.current_stream()
    out = {"batch": args.batch, "mode": args.mode, "instances": len(progs), "streams": args.streams}
    t0 = time.perf_counter()
    ex = batch.BatchExecutor(progs, mode, nstreams=args.streams)
    out["build_s"] = time.perf_counter() - t0
    ms = time_steps(ex, args.steps, args.warmup, stream)
    counts = ex.counts(stream)
    work = ex.work()
    ex.close()
    have = ~np.isnan(refs)
    full, prefix = reference_errors(progs, items, counts, mode, stream=stream)
    rel = np.concatenate([full, prefix])
    out.update({"ms_per_step": ms, "counts_per_s": len(progs) * 1e3 / ms,
                "executed_tflops": work["executed_flops"] / (ms * 1e-3) / 1e12,
                "slices": work["slices"], "checked_against_reference": int(rel.size),
                "checked_full_count": int(full.size), "checked_slice_prefix": int(prefix.size),
                "max_rel_err": float(rel.max()) if rel.size else None})
    if args.tune:
        tuner = batch.Autotuner(mode)
        t0 = time.perf_counter()
        shapes = tuner.tune(progs[:args.tune], repeats=1)
        tune_s = time.perf_counter() - t0
        ex = batch.BatchExecutor(progs, mode, nstreams=args.streams, tuner=tuner)
        ms_t = time_steps(ex, args.steps, args.warmup, stream)
        counts_t = ex.counts(stream)
        applied = ex.kernels_applied
        ex.close()
        rel_t = np.abs(counts_t[have] - refs[have]) / np.abs(refs[have])
        out["autotuned"] = {"tuned_on": args.tune, "shapes": shapes, "tune_s": tune_s, "kernels_set": applied,
                            "ms_per_step": ms_t, "counts_per_s": len(progs) * 1e3 / ms_t,
                            "max_rel_err": float(rel_t.max()) if rel_t.size else None,
                            "max_rel_diff_vs_untuned": float(np.max(np.abs(counts_t - counts) / np.abs(counts)))}
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
