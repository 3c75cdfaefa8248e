"""The learned cost model end to end on the GPU: timings the backend records
itself, training with the device kernels, and the selector's choice of slice
set and kernels.  Whatever it chooses, the count is the reference's (split
form, 1e-6); the chosen configuration must not run slower than the FLOP-model
choice beyond timing noise, and the measured times of both are reported."""
import numpy as np
import pytest

from conftest import load_golden
from tensororder_gb300 import costmodel, learned, runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu

MODE = runtime.MODE_SPLIT


def prog(name):
    return Program.from_dict(load_golden(name)["program"])


def test_recorded_timings_cover_every_allowed_kernel(cuda):
    p = prog("wvc120")
    rows = learned.record_timings(p, MODE, repeats=1)
    table = costmodel.join_table(p)
    want = sum(len(learned.allowed_kernels_host(j, MODE)) for j in table)
    assert len(rows) == want
    assert all(r.ms > 0 for r in rows)
    assert all(r.features.shape == (learned.NUM_FEATURES,) for r in rows)


def test_host_kernel_rules_match_the_library(cuda):
    for name in ("wvc120", "r3cnf20_factor", "wvc40_early"):
        p = prog(name)
        dp = runtime.DeviceProgram(p)
        lib_rules = dp.allowed_kernels(MODE)
        dp.close()
        host_rules = [learned.allowed_kernels_host(j, MODE) for j in costmodel.join_table(p)]
        assert lib_rules == host_rules


def test_selector_changes_only_speed(cuda):
    train = []
    for name in ("wvc120", "vc60_s4", "wvc30_s3", "r3cnf20_factor", "vc50_seed0"):
        for cand in costmodel.slice_candidates(prog(name), 0, 3):
            train += learned.record_timings(cand, MODE, repeats=1)
    model = learned.LearnedCostModel(seed=1)
    losses = model.fit(train, epochs=1500)
    assert losses[-1] < losses[0]
    held_out = prog("wvc40_early")
    want = float(load_golden("wvc40_early")["reference"]["float64"])
    cands = costmodel.slice_candidates(held_out, 0, 4)
    wb = learned.workspace_per_slice(cands, MODE)
    sel = learned.Selector(MODE, model)
    mine = sel.choose(cands, wb)
    base = sel.choose_flop_model(cands, wb)
    assert mine.method == "learned" and base.method == "flop-model"
    c1, t1 = learned.run_choice(mine, MODE, repeats=5)
    c0, t0 = learned.run_choice(base, MODE, repeats=5)
    assert abs(c1 - want) <= 1e-6 * want and abs(c0 - want) <= 1e-6 * want
    print("learned choice %.3f ms (%d slices), FLOP-model choice %.3f ms (%d slices)"
          % (t1 * 1e3, mine.program.num_slices, t0 * 1e3, base.program.num_slices))
    assert t1 <= 1.25 * t0 + 2e-4


def test_untrained_model_falls_back_to_flop_model(cuda):
    cands = costmodel.slice_candidates(prog("wvc120"), 0, 2)
    sel = learned.Selector(MODE, learned.LearnedCostModel())
    ch = sel.choose(cands, learned.workspace_per_slice(cands, MODE))
    assert ch.method == "flop-model"
