"""The learned cost model end to end on the GPU: timings the backend records
itself, training with the device kernels, and the selector's choice of slice
set and kernels.  Whatever it chooses, the count is the reference's (split
form, 1e-6).  On held-out random 3-CNF instances the learned choices must
save at least 5% of the summed count time against the FLOP/memory model's
choices; the measured times of both are reported."""
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


def _batch_3cnf(lo=3e11, hi=2e13):
    """Random 3-CNF instances of the 512-instance batch with 3e11..2e13
    executed FLOP per count, by index."""
    import gzip
    import json
    import os

    from conftest import ROOT

    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", "batch512.json.gz"), "rt") as f:
        items = json.load(f)["instances"]
    pool = [it for it in items if it["kind"] == "random_3cnf" and lo <= it["executed_flops"] <= hi]
    return sorted(pool, key=lambda it: it["index"])


def _slice_sets(it):
    """The instance's tree sliced 0..10 groups deep along the reference's
    greedy order, keeping the candidates whose tensors have rank <= 28."""
    p = Program.from_dict(it["program"])
    base = Program(p.leaves, p.postorder, [])
    return [c for c in costmodel.slice_candidates(base, 0, 10) if costmodel.max_rank(c) <= 28]


def test_learned_selector_beats_flop_model_on_held_out_instances(cuda):
    """What the trained network gains over the method without it.

    Training rows are the backend's own per-join timings (default kernels) of
    every slice set of ten random 3-CNF batch instances (index = 1 mod 4).
    On ten held-out instances (index = 3 mod 4) the learned selector and the
    FLOP/memory model each pick a slice set; both are contracted in full and
    timed.  The FLOP model prices every FLOP alike, while the joins that
    appear when these trees are sliced deep run far below the tensor-core
    rate, so it can pick a slicing that measures much slower.  The learned
    choice must save at least 5% of the summed count time, and both choices
    must give the same count (1e-6)."""
    pool = _batch_3cnf()
    train = [it for it in pool if it["index"] % 4 == 1][:10]
    held = [it for it in pool if it["index"] % 4 == 3][:10]
    assert len(train) == 10 and len(held) == 10
    rows = []
    for it in train:
        for cand in _slice_sets(it):
            rows += learned.record_timings(cand, MODE, kernels=(-1,), repeats=1)
    model = learned.LearnedCostModel(seed=1)
    losses = model.fit(rows, epochs=1500, batch=4096)
    assert losses[-1] < 0.1 * losses[0]
    sel = learned.Selector(MODE, model, kernels=())  # slice sets only; every join on its default kernel
    t_learned = t_flop = 0.0
    for it in held:
        cands = _slice_sets(it)
        wb = learned.workspace_per_slice(cands, MODE)
        mine, base = sel.choose(cands, wb), sel.choose_flop_model(cands, wb)
        assert mine.method == "learned" and all(k == -1 for k in mine.kernels)
        c1, t1 = learned.run_choice(mine, MODE, repeats=5)
        c0, t0 = learned.run_choice(base, MODE, repeats=5)
        assert abs(c1 - c0) <= 1e-6 * abs(c0)
        print("instance %d: learned %d groups %.3f ms, FLOP model %d groups %.3f ms"
              % (it["index"], len(mine.program.slice_groups), t1 * 1e3, len(base.program.slice_groups), t0 * 1e3))
        t_learned += t1
        t_flop += t0
    gain = t_flop / t_learned
    print("held-out total: learned %.2f ms, FLOP model %.2f ms, gain %.3fx" % (t_learned * 1e3, t_flop * 1e3, gain))
    assert gain >= 1.05


def test_untrained_model_falls_back_to_flop_model(cuda):
    cands = costmodel.slice_candidates(prog("wvc120"), 0, 2)
    sel = learned.Selector(MODE, learned.LearnedCostModel())
    ch = sel.choose(cands, learned.workspace_per_slice(cands, MODE))
    assert ch.method == "flop-model"
