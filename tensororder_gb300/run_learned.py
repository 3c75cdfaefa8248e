"""The learned cost model against the FLOP/memory model, on the GPU.

    python -m tensororder_gb300.run_learned [--epochs E] [--sample S] [--out PATH]

1. Records per-launch timings of every kernel each join may run (the
   backend's own CUDA-event timing) on training programs:
   * config-2 style GEMM joins: two seeded dense intermediates contracted with
     random extents (``tests``-independent generator below), small ones under
     every kernel and large ones (M, N of 2^12..2^14, K of 2^8..2^12) on their
     default kernels,
   * slice candidates of the n=220 weighted cubic vertex-cover plan,
   * instances of the 512-instance uneven batch.
2. Trains the MLP (the package's own forward/backward/Adam kernels).
3. For two held-out plans it lets the learned selector and the FLOP-model
   selector each choose a slice set and kernels:
   * n=220 (``wvc220_s10``, unsliced tree, candidates with 8..13 groups): both
     choices are contracted in full; the counts must equal the reference's.
   * n=300 (``wvc300``, candidates from its own slicing upwards): one count is
     ~5.5e16 FLOP, so each choice is timed on 1 and 2 slices and extrapolated
     as ``t(1) + (S - 1) * (t(2) - t(1))``.
Prints one JSON line with the choices, predicted and measured times and the
gain (FLOP-model time / learned time).
"""
from __future__ import annotations

import argparse
import gzip
import json
import os
import sys
import time

import numpy as np

from . import costmodel, learned, runtime
from .program import Leaf, Program

HERE = os.path.dirname(os.path.abspath(__file__))
MODE = runtime.MODE_SPLIT


def gemm_program(seed, m, n, k):
    """Two dense intermediates X (free m | shared k) and Y (shared k | free n),
    each the outer product of two seeded leaves, joined over k."""
    rng = np.random.default_rng(seed)
    edges = list(range(m + n + k))
    fa, fb, kk = edges[:m], edges[m:m + n], edges[m + n:]
    leaves = []
    for axes in (list(rng.permutation(fa + kk)), list(rng.permutation(kk + fb))):
        cut = len(axes) // 2
        for h in (axes[:cut], axes[cut:]):
            leaves.append(Leaf([int(e) for e in h], "dense", values=rng.uniform(0.5, 1.5, size=(2,) * len(h))))
    return Program(leaves, [0, 1, -1, 2, 3, -1, -1]).validate()


def load_workload(name):
    with gzip.open(os.path.join(HERE, "plans", name + ".json.gz"), "rt") as f:
        doc = json.load(f)
    return Program.from_dict(doc["program"]), doc["reference"]["float64"]


def training_rows(batch_instances=16, gemm_programs=16, big_gemm_programs=8, seed=0):
    rows = []
    rng = np.random.default_rng(seed)
    for i in range(gemm_programs):
        m, n, k = (int(x) for x in rng.integers(6, 12, size=3))
        k = int(rng.integers(2, 11))
        rows += learned.record_timings(gemm_program(1000 + i, m, n, k), MODE, repeats=2)
    # Joins of the size n=300's plans hold (up to 2^28 outputs, K up to 2^12), on
    # their default kernels only: the thread-per-output kernel would take minutes.
    for i in range(big_gemm_programs):
        m, n = (int(x) for x in rng.integers(12, 15, size=2))
        k = int(rng.integers(8, 13))
        rows += learned.record_timings(gemm_program(2000 + i, m, n, k), MODE, kernels=(-1,), repeats=2)
    p220, _ = load_workload("wvc220_s10")
    base = Program(p220.leaves, p220.postorder, [])
    for cand in costmodel.slice_candidates(base, 10, 12):
        rows += learned.record_timings(cand, MODE, repeats=2)
    with gzip.open(os.path.join(HERE, "plans", "batch512.json.gz"), "rt") as f:
        items = json.load(f)["instances"]
    for it in items[:batch_instances]:
        if it["executed_flops"] < 1e12:
            rows += learned.record_timings(Program.from_dict(it["program"]), MODE, repeats=1)
    return rows


def describe(choice):
    ks = [k for k in choice.kernels if k >= 0]
    return {"method": choice.method, "slice_groups": len(choice.program.slice_groups),
            "slices": choice.program.num_slices, "predicted_s": choice.predicted_s,
            "kernels_set": len(ks), "kernels_by_id": {str(k): ks.count(k) for k in sorted(set(ks))}}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)

    t0 = time.perf_counter()
    rows = training_rows()
    t_rec = time.perf_counter() - t0
    model = learned.LearnedCostModel(seed=0)
    t0 = time.perf_counter()
    losses = model.fit(rows, epochs=args.epochs)
    t_fit = time.perf_counter() - t0
    X = np.stack([r.features for r in rows])
    y = np.array([r.ms for r in rows])
    pred = model.predict_ms(X)
    out = {"training_rows": len(rows), "record_s": t_rec, "fit_s": t_fit, "loss_first": losses[0],
           "loss_last": losses[-1],
           "train_median_abs_log_err": float(np.median(np.abs(np.log(pred) - np.log(y))))}
    if args.out:
        model.save(args.out)
    sel = learned.Selector(MODE, model)

    # n=220: full counts of both choices.
    p220, ref220 = load_workload("wvc220_s10")
    base = Program(p220.leaves, p220.postorder, [])
    cands = costmodel.slice_candidates(base, 8, 13)
    wb = learned.workspace_per_slice(cands, MODE)
    mine, flop = sel.choose(cands, wb), sel.choose_flop_model(cands, wb)
    c1, t1 = learned.run_choice(mine, MODE, repeats=5)
    c0, t0_ = learned.run_choice(flop, MODE, repeats=5)
    out["wvc220"] = {"learned": dict(describe(mine), measured_s=t1, rel_err=abs(c1 - ref220) / ref220),
                     "flop_model": dict(describe(flop), measured_s=t0_, rel_err=abs(c0 - ref220) / ref220),
                     "gain": t0_ / t1}

    # n=300: sampled slices, extrapolated.
    with gzip.open(os.path.join(HERE, "plans", "wvc300.json.gz"), "rt") as f:
        p300 = Program.from_dict(json.load(f)["program"])
    g0 = len(p300.slice_groups)
    base = Program(p300.leaves, p300.postorder, [])
    cands = costmodel.slice_candidates(base, g0, g0 + 4)
    wb = learned.workspace_per_slice(cands, MODE)
    res = {}
    for ch in (sel.choose(cands, wb), sel.choose_flop_model(cands, wb)):
        _, ta = learned.run_choice(ch, MODE, repeats=2, max_slices=1, max_fraction=0.8)
        _, tb = learned.run_choice(ch, MODE, repeats=2, max_slices=2, max_fraction=0.8)
        est = ta + (ch.program.num_slices - 1) * max(0.0, tb - ta)
        res[ch.method] = dict(describe(ch), sample_s=[ta, tb], extrapolated_s=est)
    res["gain"] = res["flop-model"]["extrapolated_s"] / res["learned"]["extrapolated_s"]
    out["wvc300"] = res
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
