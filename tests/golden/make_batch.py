"""Freeze an uneven batch of seeded instances with their own plans
(``togb.batch/1``, one gzipped JSON document).

Needs the reference checkout and ``python oracle/build_ref.py``.  Instance
``i`` of the batch (seed ``base_seed + i``):

* even ``i``: weighted cubic vertex cover of a seeded random 3-regular graph
  with ``n ~ U{30..160}`` (rounded to even), cachet weights ``p ~ U(0.2, 0.8)``,
  planned with line-Flow;
* odd ``i``: random 3-CNF with ``v ~ U{40..v_max}`` variables and
  ``floor(1.8 v)`` clauses of three distinct variables with random polarity,
  cachet weights ``p ~ U(0.2, 0.8)``, planned with factor-Flow.  ``v_max`` is 52:
  above it the reference's planners (a few seconds each) give plans of
  1e13-1e19 FLOPs per count, too large for one batch step.

Each plan is then sliced by the reference's greedy memory slicer until it has
``g ~ U{0..8}`` slice groups (1 to 2^8 slices) and every tensor has rank <= 30.
The reference's numpy FP64 count is recorded for instances whose executed work
is below ``ref_flops`` (others carry ``null``; their parity is checked between
the two GPU forms).

Usage: ``python tests/golden/make_batch.py [count] [out]``.
"""
import contextlib
import gzip
import io
import json
import os
import random
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PLANS = os.path.join(ROOT, "tensororder_gb300", "plans")
sys.path.insert(0, ROOT)

from oracle import refload  # noqa: E402
from tensororder_gb300 import costmodel, instances  # noqa: E402
from tensororder_gb300.program import from_plan  # noqa: E402


def instance_plan(i, base_seed=1000, v_max=52, timeout=1.0):
    """The reference plan of instance ``i``: ``(kind, size, planner, plan)``."""
    seed = base_seed + i
    rng = random.Random(seed)
    g = rng.randint(0, 8)
    if i % 2 == 0:
        n = 2 * (rng.randint(30, 160) // 2)
        cnf = instances.cubic_vertex_cover_cnf(n, seed, weighted=True, lo=0.2, hi=0.8)
        kind, size, planner = "cubic_vc", n, "line-Flow"
    else:
        v = rng.randint(40, v_max)
        cnf = instances.random_3cnf(v, 1.8, seed, weighted=True, lo=0.2, hi=0.8)
        kind, size, planner = "random_3cnf", v, "factor-Flow"
    sink = io.StringIO()
    with contextlib.redirect_stdout(sink), contextlib.redirect_stderr(sink):
        plan = refload.plan_cnf(cnf, weights="cachet", planner=planner, seed=0, timeout=timeout,
                                minimum_slice=g, rank_limit=30)
    return kind, size, planner, plan


def make_instance(i, base_seed=1000, v_max=52, timeout=1.0, ref_flops=2e9):
    seed = base_seed + i
    kind, size, planner, plan = instance_plan(i, base_seed, v_max, timeout)
    sink = io.StringIO()
    prog = from_plan(plan)
    cost = costmodel.executed_cost(prog)
    ref = None
    if cost["flops"] <= ref_flops:
        with contextlib.redirect_stdout(sink), contextlib.redirect_stderr(sink):
            ref = float(refload.reference_count(plan))
    return {"index": i, "seed": seed, "kind": kind, "size": size, "planner": planner,
            "slice_groups": len(prog.slice_groups), "executed_flops": cost["flops"],
            "program": prog.to_dict(), "reference_float64": ref}


def main():
    count = int(sys.argv[1]) if len(sys.argv) > 1 else 512
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(PLANS, "batch%d.json.gz" % count)
    t0 = time.time()
    items = []
    for i in range(count):
        items.append(make_instance(i))
        if (i + 1) % 32 == 0:
            print("%d/%d instances, %.0f s" % (i + 1, count, time.time() - t0), flush=True)
    doc = {"format": "togb.batch/1", "count": count, "instances": items}
    data = json.dumps(doc, separators=(",", ":")).encode()
    with open(out, "wb") as f:
        f.write(gzip.compress(data, mtime=0))
    print("wrote", out, len(data), "bytes raw")


if __name__ == "__main__":
    main()
