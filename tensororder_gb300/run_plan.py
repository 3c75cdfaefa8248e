"""Contract a frozen plan on the GPU and report its count and device time.

    python -m tensororder_gb300.run_plan PLAN [--mode split|f64] [--slices N]
                                              [--repeat R] [--joins]

``PLAN`` is a ``togb.workload/1`` file (``tensororder_gb300/plans/*.json.gz``,
carrying the reference's own count) or a ``togb.program/1`` file.  The first
``N`` slices (default: all) are contracted ``R`` times; with ``--joins`` one
more pass records the device time of every join with CUDA events and prints
the joins sorted by time.  This is the small-case driver for profiling single
kernels: ``--slices`` bounds the device memory and the launch sizes.
"""
from __future__ import annotations

import argparse
import gzip
import json
import sys

import numpy as np

from . import runtime
from .program import Program


def load(path):
    opener = gzip.open if path.endswith(".gz") else open
    with opener(path, "rt") as f:
        doc = json.load(f)
    if doc.get("format") == "togb.workload/1":
        return Program.from_dict(doc["program"]), doc.get("reference", {}).get("float64")
    return Program.from_dict(doc), None


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("plan")
    ap.add_argument("--mode", choices=["split", "f64"], default="split")
    ap.add_argument("--slices", type=int, default=None)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--joins", action="store_true")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)

    import torch

    prog, ref = load(args.plan)
    mode = runtime.MODE_SPLIT if args.mode == "split" else runtime.MODE_F64
    dp = runtime.DeviceProgram(prog, args.device)
    n = dp.num_slices if args.slices is None else min(dp.num_slices, args.slices)
    ws = dp.allocate_workspace(mode, n, max_fraction=0.6)
    stream = torch.cuda.current_stream(args.device)
    ms = []
    for _ in range(max(1, args.repeat)):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        dp.reset(stream)
        a.record(stream)
        dp.run(mode, 0, n, workspace=ws, stream=stream)
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
    count = float(dp.result(stream).reshape(-1)[0])
    out = {"plan": args.plan, "mode": args.mode, "slices": n, "count": count, "ms": ms}
    if ref is not None and n == dp.num_slices:
        out["rel_err_vs_reference"] = abs(count - ref) / abs(ref)
    print(json.dumps(out))
    if args.joins:
        dp.set_timing(True)
        dp.reset(stream)
        dp.run(mode, 0, n, workspace=ws, stream=stream)
        torch.cuda.synchronize(args.device)
        t = dp.join_times()
        info = dp.joins(mode)
        order = np.argsort(-t)
        print("join  log2(M,N,K)  kernel  per_slice  ms")
        for j in order:
            mb, nb, kb, kern, per = (int(x) for x in info[j])
            print("%4d  (%2d,%2d,%2d)  %-7s %-9s %.4f" % (j, mb, nb, kb, runtime.KERNEL_NAMES[kern],
                                                       "yes" if per else "once", t[j]))
    dp.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
