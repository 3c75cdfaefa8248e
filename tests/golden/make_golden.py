"""Generate the golden fixtures in ``tests/golden/`` by running the reference.

Requires the reference checkout and ``python oracle/build_ref.py``.  For each
case it:

1. writes a seeded synthetic CNF (or reads the reference's bundled instance),
2. runs the reference's own Reduction + Planning + Slicing
   (``oracle.refload.plan_cnf``: ``cnf_count``, ``planning.run`` with
   FlowCutter, ``slicer.slice_until``),
3. freezes the plan as a ``togb.program/1`` document
   (``tensororder_gb300.program.from_plan``),
4. contracts the plan with the reference's numpy backend
   (``numpy_apis.py`` via ``base_api.contract_sliced``) in float64 -- and in
   ``bigint`` for unweighted cases -- and, for small instances, by brute force
   over all assignments.

Planning is anytime and timing-dependent, so the frozen plan (not the seed) is
what the fixtures pin; regenerating may give different plans with the same
counts.  Usage: ``python tests/golden/make_golden.py [case ...]``.
"""
import io
import itertools
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refload  # noqa: E402
from tensororder_gb300 import instances  # noqa: E402
from tensororder_gb300.program import from_plan  # noqa: E402


def brute_force(cnf_text, weights):
    """Weighted model count by enumerating every assignment (n <= 22)."""
    nv, clauses, w = instances.parse_cnf(cnf_text)
    if nv > 22:
        return None
    default = (0.5, 0.5) if weights == "cachet" else (1.0, 1.0)
    bits = (np.arange(1 << nv, dtype=np.int64)[:, None] >> np.arange(nv)[None, :]) & 1
    ok = np.ones(1 << nv, dtype=bool)
    for c in clauses:
        sat = np.zeros(1 << nv, dtype=bool)
        for lit in c:
            col = bits[:, abs(lit) - 1]
            sat |= (col == 1) if lit > 0 else (col == 0)
        ok &= sat
    val = np.ones(1 << nv, dtype=np.float64)
    for v in range(1, nv + 1):
        wn, wp = w.get(v, default)
        val *= np.where(bits[:, v - 1] == 1, wp, wn)
    return float(val[ok].sum())


CASES = {
    # Reference's bundled instance (benchmarks/cubic_vertex_cover/cubic_vc_50_0.cnf).
    "vc50_bundled": dict(cnf="bundled", weights="unweighted", planner="line-Flow", timeout=3),
    # Seeded n=50 unweighted cubic vertex cover, line-Flow, no slicing.
    "vc50_seed0": dict(cnf=("vc", 50, 0, False), weights="unweighted", planner="line-Flow", timeout=3),
    # Small weighted, sliced into 8 slices: pins slice order via prefix counts.
    "wvc30_s3": dict(cnf=("vc", 30, 1, True), weights="cachet", planner="line-Flow", timeout=2,
                     minimum_slice=3, prefixes=True),
    "wvc18_s2": dict(cnf=("vc", 18, 5, True), weights="cachet", planner="line-Flow", timeout=1,
                     minimum_slice=2, prefixes=True),
    # Unweighted sliced, exact bigint count.
    "vc60_s4": dict(cnf=("vc", 60, 3, False), weights="unweighted", planner="line-Flow", timeout=3,
                    minimum_slice=4),
    # factor-Flow: factored OR gates (output_index) and (1,1) variable tensors.
    "r3cnf20_factor": dict(cnf=("r3", 20, 1.8, 2), weights="cachet", planner="factor-Flow", timeout=2,
                           minimum_slice=2),
    "r3cnf16_line": dict(cnf=("r3", 16, 1.8, 7), weights="cachet", planner="line-Flow", timeout=1),
    # --early: contract_small turns low-rank subtrees into dense BuiltTensor leaves.
    "wvc40_early": dict(cnf=("vc", 40, 11, True), weights="cachet", planner="line-Flow", timeout=2,
                        early=6, minimum_slice=2),
    # Larger unsliced weighted case (max rank ~14) for the GEMM path.
    "wvc120": dict(cnf=("vc", 120, 4, True), weights="cachet", planner="line-Flow", timeout=6),
}


def make_cnf(spec):
    if spec == "bundled":
        path = os.path.join(refload.reference_src(), "..", "benchmarks", "cubic_vertex_cover", "cubic_vc_50_0.cnf")
        with open(path) as f:
            return f.read()
    if spec[0] == "vc":
        _, n, seed, weighted = spec
        return instances.cubic_vertex_cover_cnf(n, seed, weighted=weighted)
    if spec[0] == "r3":
        _, v, ratio, seed = spec
        return instances.random_3cnf(v, ratio, seed)
    raise ValueError(spec)


def make_case(name, spec):
    ref = refload.load()
    cnf = make_cnf(spec["cnf"])
    plan = refload.plan_cnf(cnf, weights=spec["weights"], planner=spec["planner"], seed=0,
                            timeout=spec["timeout"], minimum_slice=spec.get("minimum_slice", 0))
    if spec.get("early"):
        # tensororder.py:273-276 runs contract_small with the numpy API.
        numpy_api = ref.tensor_network.ALL_APIS["numpy"]()
        numpy_api.add_argument("entry_type", "float64")
        plan.contract_small(spec["early"], numpy_api)
    prog = from_plan(plan)
    doc = {
        "format": "togb.workload/1",
        "name": name,
        "cnf": cnf,
        "weights": spec["weights"],
        "planner": spec["planner"],
        "minimum_slice": spec.get("minimum_slice", 0),
        "early": spec.get("early", 0),
        "program": prog.to_dict(),
        "reference": {"float64": float(refload.reference_count(plan))},
    }
    if spec["weights"] == "unweighted":
        doc["reference"]["bigint"] = str(int(refload.reference_count(plan, "bigint")))
    if spec.get("prefixes"):
        doc["reference"]["prefix_float64"] = [
            float(refload.reference_count(plan, num_slice_limit=k)) for k in range(1, prog.num_slices + 1)
        ]
    if not spec.get("early"):
        bf = brute_force(cnf, spec["weights"])
        if bf is not None:
            doc["brute_force"] = bf
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(doc, f, separators=(",", ":"))
        f.write("\n")
    print(name, prog.num_joins, "joins", prog.num_slices, "slices", doc["reference"], doc.get("brute_force"))


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for n in names:
        make_case(n, CASES[n])
