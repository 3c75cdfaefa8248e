"""Freeze oracle counts of single slices of the n=300 workload, sliced deep.

One slice of ``plans/wvc300.json.gz`` at its own slicing (9 groups, rank 30)
is about 1e14 FLOP with 2^30-entry tensors, beyond a CPU contraction here.
The same contraction tree sliced 22 groups deep along the reference's greedy
order (``costmodel.greedy_slice_sequence``) has slices of 5.6e10 FLOP at rank
24, which ``oracle/contract.py`` (the reference's numpy execution restated)
contracts in a few seconds each.  The slice sets partition the same sum, so a
slice of the deep slicing is a piece of the n=300 count: the GPU must
reproduce it in both forms.

Slices: the last three (every sliced vertex in the cover, so no clause can be
falsified and the counts are nonzero) and three seeded ones.  The 22 groups
are stored with the counts, so the test does not depend on the slicer.

Usage: ``python tests/golden/make_wvc300_slices.py`` (writes
``tests/golden/slices/wvc300.json``).
"""
import gzip
import json
import os
import random
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import contract as oracle  # noqa: E402
from tensororder_gb300 import costmodel  # noqa: E402
from tensororder_gb300.program import Program  # noqa: E402

GROUPS = 22


def main():
    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", "wvc300.json.gz"), "rt") as f:
        prog = Program.from_dict(json.load(f)["program"])
    base = Program(prog.leaves, prog.postorder, [])
    groups = costmodel.greedy_slice_sequence(base, GROUPS)[:GROUPS]
    deep = costmodel.with_groups(base, groups)
    S = deep.num_slices
    rng = random.Random(300)
    slices = [S - 3, S - 2, S - 1] + sorted(rng.randrange(S) for _ in range(3))
    out = []
    t0 = time.time()
    for s in slices:
        v, _ = oracle.contract(deep, s)
        out.append({"slice": s, "oracle_float64": float(v)})
        print("slice %d: %r (%.0f s)" % (s, float(v), time.time() - t0), flush=True)
    doc = {"format": "togb.slices/1", "workload": "wvc300", "groups": [sorted(g) for g in groups],
           "num_slices": S, "max_rank": costmodel.max_rank(deep), "slices": out}
    with open(os.path.join(HERE, "slices", "wvc300.json"), "w") as f:
        json.dump(doc, f, indent=1)


if __name__ == "__main__":
    main()
