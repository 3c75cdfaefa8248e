"""The cost model restatement against the reference's own figures
(tests/golden/cost/*.json, made by tests/golden/make_cost_golden.py):
FLOPs, memory cap, next edge to slice and max rank after every step of the
reference's greedy memory slicer, and the groups that slicer picks."""
import glob
import json
import os

import pytest

from conftest import GOLDEN_DIR, load_golden
from tensororder_gb300 import costmodel
from tensororder_gb300.program import Program

COST = sorted(glob.glob(os.path.join(GOLDEN_DIR, "cost", "*.json")))


def load(path):
    with open(path) as f:
        doc = json.load(f)
    return Program.from_dict(doc["program"]), doc["steps"]


@pytest.mark.parametrize("path", COST, ids=[os.path.basename(p)[:-5] for p in COST])
def test_estimate_matches_reference_along_greedy_slicing(path):
    prog, steps = load(path)
    for st in steps:
        sliced = {e for g in st["groups"] for e in g}
        info = costmodel.reference_estimate(prog, sliced)
        assert info.flops == st["flops"]
        assert info.total_memory == st["memory"]
        assert info.largest_tensor == st["max_rank"]
        assert info.best_edge == st["next_edge"]


@pytest.mark.parametrize("path", COST, ids=[os.path.basename(p)[:-5] for p in COST])
def test_greedy_sequence_matches_reference_slicer(path):
    prog, steps = load(path)
    seq = costmodel.greedy_slice_sequence(prog, max_groups=len(steps) - 1)
    want = steps[-1]["groups"]
    assert [sorted(g) for g in seq] == [sorted(g) for g in want]


def test_executed_cost_counts_invariant_joins_once():
    prog = Program.from_dict(load_golden("wvc30_s3")["program"])
    c = costmodel.executed_cost(prog)
    js = costmodel.join_table(prog)
    assert c["slices"] == 8
    per = sum(j.flops for j in js if j.per_slice)
    once = sum(j.flops for j in js if not j.per_slice)
    assert c["flops"] == per * 8 + once
    assert c["flops_reference_order"] == (per + once) * 8
    assert js[-1].per_slice


def test_slice_candidates_are_valid_programs_with_growing_slices():
    prog = Program.from_dict(load_golden("wvc120")["program"])
    cands = costmodel.slice_candidates(prog, 0, 6)
    assert [c.num_slices for c in cands] == [1 << k for k in range(len(cands))]
    ranks = [costmodel.max_rank(c) for c in cands]
    assert ranks == sorted(ranks, reverse=True)
