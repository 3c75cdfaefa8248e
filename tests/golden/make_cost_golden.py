"""Generate ``tests/golden/cost/*.json``: the reference's own cost-model
figures along its greedy slicing sequence.

Requires the reference checkout and ``python oracle/build_ref.py``.  For each
case it plans a seeded instance with the reference's planner, freezes the
unsliced plan as a ``togb.program/1`` document, then applies the reference's
``GreedyMemSlicer`` one group at a time (``slicers.py:27-33`` ->
``SlicedExecutionPlan.slice_at``, ``sliced_execution_plan.py:58-82``) and
records after every step what ``ContractionTree.estimate_cost``
(``contraction_methods/contraction_tree.pyx:382-496``) reported: FLOPs, memory
cap, next edge to slice, max rank, and the groups sliced so far.

Usage: ``python tests/golden/make_cost_golden.py``.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refload  # noqa: E402
from tensororder_gb300 import instances  # noqa: E402
from tensororder_gb300.program import from_plan  # noqa: E402

CASES = {
    "wvc60": dict(kind="vc", n=60, seed=2, planner="line-Flow", steps=8),
    "wvc120": dict(kind="vc", n=120, seed=4, planner="line-Flow", steps=10),
    "r3cnf30_factor": dict(kind="r3", n=30, seed=3, planner="factor-Flow", steps=6),
}


def make(name):
    spec = CASES[name]
    if spec["kind"] == "vc":
        cnf = instances.cubic_vertex_cover_cnf(spec["n"], spec["seed"], weighted=True)
    else:
        cnf = instances.random_3cnf(spec["n"], 1.8, spec["seed"])
    plan = refload.plan_cnf(cnf, weights="cachet", planner=spec["planner"], seed=0, timeout=3,
                            minimum_slice=0, rank_limit=64)
    prog = from_plan(plan)
    ref = refload.load()
    slicer = ref.tensor_network.ALL_SLICERS["greedy_mem"]
    steps = []
    for _ in range(spec["steps"] + 1):
        steps.append({
            "groups": [sorted(int(e) for e in g) for g in plan.groups_to_slice],
            "flops": float(plan.FLOPs), "memory": float(plan.memory),
            "next_edge": int(plan.next_edge_to_slice), "max_rank": int(plan.maxrank),
        })
        slicer.slice_once(plan)
    doc = {"format": "togb.costgolden/1", "name": name, "program": prog.to_dict(), "steps": steps}
    with open(os.path.join(HERE, "cost", name + ".json"), "w") as f:
        json.dump(doc, f, separators=(",", ":"))
    print(name, prog.num_joins, "joins", len(steps), "steps")


if __name__ == "__main__":
    for n in sys.argv[1:] or list(CASES):
        make(n)
