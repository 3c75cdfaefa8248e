"""Freeze the benchmark workloads as ``togb.workload/1`` documents.

Needs the reference checkout and ``python oracle/build_ref.py`` (FlowCutter and
the reference's Cython).  Each workload records the CNF, the frozen plan and
the reference's own numpy FP64 count on that plan, so the GPU runs need neither
the reference nor a planner.

* ``wvc220_s10`` -- weighted cubic vertex cover, seeded random 3-regular graph
  with n=220 vertices (330 edge clauses), cachet weights p ~ U(0.3, 0.7),
  line-Flow plan sliced with ``--minimum_slice 10`` into 2^10 equal-shape
  slices.
* ``wvc300`` -- the same construction with n=300, sliced only as rank 30
  requires (the held-out instance of the learned cost model).

Usage: ``python tests/golden/make_plans.py [name ...]``.
"""
import gzip
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PLANS = os.path.join(ROOT, "tensororder_gb300", "plans")
sys.path.insert(0, ROOT)

from oracle import refload  # noqa: E402
from tensororder_gb300 import instances  # noqa: E402
from tensororder_gb300.program import from_plan  # noqa: E402

WORKLOADS = {
    "wvc220_s10": dict(n=220, seed=0, weights="cachet", planner="line-Flow", timeout=20, minimum_slice=10),
    # Held-out instance of the learned cost model: weighted cubic vertex cover,
    # n=300 (450 edge clauses), seed 0, line-Flow, sliced only as far as rank 30
    # requires.  Its count is ~5.5e16 FLOP, beyond a CPU reference run, so the
    # document records no reference count.
    "wvc300": dict(n=300, seed=0, weights="cachet", planner="line-Flow", timeout=60, minimum_slice=0,
                   reference=False),
}


def make(name):
    spec = WORKLOADS[name]
    cnf = instances.cubic_vertex_cover_cnf(spec["n"], spec["seed"], weighted=spec["weights"] == "cachet")
    plan = refload.plan_cnf(cnf, weights=spec["weights"], planner=spec["planner"], seed=0,
                            timeout=spec["timeout"], minimum_slice=spec["minimum_slice"])
    prog = from_plan(plan)
    t = time.time()
    count = float(refload.reference_count(plan)) if spec.get("reference", True) else None
    elapsed = time.time() - t
    doc = {
        "format": "togb.workload/1",
        "name": name,
        "cnf": cnf,
        "weights": spec["weights"],
        "planner": spec["planner"],
        "minimum_slice": spec["minimum_slice"],
        "program": prog.to_dict(),
        "reference": {"float64": count, "seconds_here": elapsed, "cores_here": os.cpu_count()},
    }
    with gzip.open(os.path.join(PLANS, name + ".json.gz"), "wt") as f:
        json.dump(doc, f, separators=(",", ":"))
    print(name, prog.num_joins, "joins", prog.num_slices, "slices", count, "%.1fs" % elapsed)


if __name__ == "__main__":
    for n in sys.argv[1:] or list(WORKLOADS):
        make(n)
