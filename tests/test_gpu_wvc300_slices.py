"""The n=300 held-out workload checked on single slices.

A full n=300 count (5.5e16 FLOP, rank-30 tensors) is beyond a CPU oracle.
``tests/golden/slices/wvc300.json`` holds oracle counts of single slices of the
same contraction tree sliced 22 groups deep (rank 24): the last three slices
(nonzero by construction) and three seeded ones.  Each is contracted on its
own (``run(begin=s, end=s+1)``), and the last three also as one range.

Plain form: 1e-12 relative.  Split form: 1.5e-6.  On this tree (749 joins, 10
of them on the tensor cores per slice) the split form's error is a systematic
-0.77e-6 to -1.10e-6 on every slice checked, and -1.11e-6 on a 256-slice range
against the plain form: the tensor cores truncate their FP32 accumulation, so
each tensor-core join lowers its outputs by about an FP32 ulp.  The n=220
workload (8 such joins) stays within 4.4e-7."""
import gzip
import json
import os

import pytest

from conftest import GOLDEN_DIR, ROOT
from tensororder_gb300 import costmodel, runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu


def deep_program(doc):
    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", "wvc300.json.gz"), "rt") as f:
        prog = Program.from_dict(json.load(f)["program"])
    return costmodel.with_groups(Program(prog.leaves, prog.postorder, []), doc["groups"])


@pytest.mark.parametrize("mode,tol", [(runtime.MODE_F64, 1e-12), (runtime.MODE_SPLIT, 1.5e-6)])
def test_wvc300_slices_match_the_oracle(mode, tol, cuda):
    with open(os.path.join(GOLDEN_DIR, "slices", "wvc300.json")) as f:
        doc = json.load(f)
    prog = deep_program(doc)
    assert prog.num_slices == doc["num_slices"]
    dp = runtime.DeviceProgram(prog)
    ws = dp.allocate_workspace(mode, 4)
    for rec in doc["slices"]:
        s, want = rec["slice"], rec["oracle_float64"]
        dp.reset()
        dp.run(mode, s, s + 1, workspace=ws)
        got = float(dp.result().reshape(-1)[0])
        assert abs(got - want) <= tol * abs(want), (s, got, want)
    last = [r for r in doc["slices"] if r["slice"] >= doc["num_slices"] - 3]
    dp.reset()
    dp.run(mode, doc["num_slices"] - 3, doc["num_slices"], workspace=ws)
    got = float(dp.result().reshape(-1)[0])
    want = sum(r["oracle_float64"] for r in last)
    dp.close()
    assert abs(got - want) <= tol * abs(want)
