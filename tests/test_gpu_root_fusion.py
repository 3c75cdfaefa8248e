"""The count's final dot product formed in its operand's epilogue.

On the n=220 workload the root join is a full contraction of two per-slice
tensors of 2^19 entries, and its right operand is a tensor-core join.  The
library then has that join's epilogue multiply its output by the other
operand (stored at the same addresses) and write per-tile FP64 partials; the
root join itself is not launched and the root kernel adds the partials in a
fixed order.  The count must equal the reference's (split form, 1e-6), be the
same bits on every run, and agree with the unfused path, which runs when the
operand join is moved to the CUDA cores.
"""
import gzip
import json
import os

import numpy as np
import pytest

from conftest import ROOT
from tensororder_gb300 import runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu

MODE = runtime.MODE_SPLIT


def workload():
    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", "wvc220_s10.json.gz"), "rt") as f:
        doc = json.load(f)
    return Program.from_dict(doc["program"]), doc["reference"]["float64"]


def test_root_dot_formed_in_its_operands_epilogue(cuda):
    prog, ref = workload()
    dp = runtime.DeviceProgram(prog)
    planned = dp.launch_count(MODE)  # before any run: every join launched
    counts = []
    for _ in range(2):
        dp.reset()
        dp.run(MODE)
        counts.append(float(dp.result().reshape(-1)[0]))
    assert dp.launch_count(MODE) == planned - 1  # the root join is not launched
    assert counts[0] == counts[1]                # fixed-order partial sums: same bits
    assert abs(counts[0] - ref) <= 1e-6 * abs(ref)
    # The root's right operand is the join just before it in post-order; on the
    # CUDA cores it stores its output and the root join runs as usual.
    x = int(dp.info.num_joins) - 2
    dp.set_kernel(MODE, x, 0)
    dp.reset()
    dp.run(MODE)
    unfused = float(dp.result().reshape(-1)[0])
    assert dp.launch_count(MODE) == planned
    assert abs(unfused - ref) <= 1e-6 * abs(ref)
    assert abs(unfused - counts[0]) <= 1e-6 * abs(ref)
    dp.close()
