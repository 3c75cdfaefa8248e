"""The fused slice-invariant phase: runs of thread-per-output joins that read
no sliced edge are executed as one launch (CTAs claiming tiles in execution
order and waiting for the tiles they read), while join-by-join timing runs
the same joins as separate launches.  Both must give the same bits: the fused
kernel follows the unfused kernels' arithmetic output by output.  Checked on
every sliced golden plan and on the n=220 workload (whose 361 slice-invariant
joins include a tensor-core join, so the phase has several fused lists), in
both forms, plus the count against the reference."""
import gzip
import json
import os

import numpy as np
import pytest

from conftest import ROOT, golden_names, load_golden
from tensororder_gb300 import runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu

SLICED = [n for n in golden_names() if Program.from_dict(load_golden(n)["program"]).slice_groups]


def run_both(prog, mode, slices=None):
    dp = runtime.DeviceProgram(prog)
    n = dp.num_slices if slices is None else min(slices, dp.num_slices)
    out = []
    launches = None
    for timing in (False, True):
        dp.set_timing(timing)
        dp.reset()
        dp.run(mode, 0, n)
        out.append(np.array(dp.result(), copy=True))
        if launches is None:
            launches = dp.launch_count(mode)
    info = dp.info
    root_fused = "fused_into_operand" in dp.describe(mode, int(info.num_joins) - 1)
    dp.close()
    return out[0], out[1], info, launches, root_fused


@pytest.mark.parametrize("name", SLICED)
@pytest.mark.parametrize("mode", [runtime.MODE_F64, runtime.MODE_SPLIT])
def test_fused_once_phase_equals_unfused(name, mode, cuda):
    doc = load_golden(name)
    prog = Program.from_dict(doc["program"])
    fused, unfused, info, _, _ = run_both(prog, mode)
    assert info.num_joins_once > 0
    assert np.array_equal(fused, unfused)
    tol = 1e-12 if mode == runtime.MODE_F64 else 1e-6
    assert abs(float(fused.reshape(-1)[0]) - doc["reference"]["float64"]) <= tol * abs(doc["reference"]["float64"])


@pytest.mark.parametrize("mode", [runtime.MODE_F64, runtime.MODE_SPLIT])
def test_fused_once_phase_equals_unfused_n220(mode, cuda):
    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", "wvc220_s10.json.gz"), "rt") as f:
        prog = Program.from_dict(json.load(f)["program"])
    fused, unfused, info, launches, root_fused = run_both(prog, mode, slices=8)
    assert info.num_joins_once == 361
    assert np.array_equal(fused, unfused)
    # A count is the slice-invariant phase, then per chunk of slices the slice
    # base, the per-slice joins (less the root join when its dot product is
    # formed in its operand's epilogue, split form) and the root: the 361
    # slice-invariant joins are queued as a handful of launches.
    assert root_fused == (mode == runtime.MODE_SPLIT)
    per_chunk = int(info.num_launches) + 1 - int(root_fused)
    assert launches // per_chunk >= 1
    assert launches % per_chunk <= 4
