"""Pin every instance of the uneven batch on a slice prefix with the
reference's own count.

``make_batch.py`` records the reference's full numpy FP64 count only for the
cheaper instances.  For every other instance this script re-runs the
reference's planner with the instance's seed and settings, checks that the
flattened plan is identical to the frozen one (FlowCutter reproduces it), and
contracts the first ``num_slice_limit`` slices with the reference's numpy
backend (``base_api.py:17-28``, ``islice`` to ``num_slice_limit`` at
``base_api.py:23-24``).  The prefix is one slice, or the whole count when the
instance has a single slice (then the full count is recorded too); when the
prefix sums to exactly zero (the first slices fix a clause false) it is doubled
until it does not, so that the GPU count can be checked to a relative
tolerance.

Each result is appended to a JSON-lines progress file as it finishes, so the
run can be stopped and resumed; ``--merge`` writes the results into the batch
document as ``reference_prefix = {"slices": P, "float64": value}``.  Cheap
instances go first.  Needs the reference checkout and
``python oracle/build_ref.py``.

Usage: ``python tests/golden/make_batch_prefix.py [--progress FILE] [--tries N]
[--timeouts S ...] [--merge]`` (the batch file was pinned with ``--tries 60
--timeouts 1.0 0.2``).
"""
import argparse
import contextlib
import gzip
import io
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_batch import PLANS, instance_plan  # noqa: E402
from oracle import refload  # noqa: E402
from tensororder_gb300.program import from_plan  # noqa: E402

BATCH = os.path.join(PLANS, "batch512.json.gz")


def load_progress(path):
    done = {}
    if os.path.exists(path):
        with open(path) as f:
            for line in f:
                if line.strip():
                    rec = json.loads(line)
                    done[rec["index"]] = rec
    return done


def pin(item, tries=1, timeouts=(1.0,)):
    """Reference count of ``item``'s first slice (or of all its slices when it
    has one).  The planner is an anytime solver under a wall-clock limit, so a
    re-plan that differs from the frozen plan is retried up to ``tries`` times
    at each planner limit of ``timeouts`` (a frozen plan the planner reached
    early under load is found again with a shorter limit)."""
    for limit in timeouts:
        for _ in range(tries):
            kind, size, planner, plan = instance_plan(item["index"], timeout=limit)
            if from_plan(plan).to_dict() == item["program"]:
                break
        else:
            continue
        break
    else:
        return {"index": item["index"], "error": "re-planned program differs from the frozen one"}
    slices = 1 << item["slice_groups"]
    prefix = 1
    t = time.time()
    sink = io.StringIO()
    while True:
        with contextlib.redirect_stdout(sink), contextlib.redirect_stderr(sink):
            value = float(refload.reference_count(plan, num_slice_limit=prefix))
        if value != 0.0 or prefix >= slices:
            break
        prefix = min(slices, 2 * prefix)
    return {"index": item["index"], "slices": prefix, "of": slices, "float64": value,
            "seconds": time.time() - t, "cores": os.cpu_count()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--progress", default=os.path.join(ROOT, "_work", "batch_prefix.jsonl"))
    ap.add_argument("--merge", action="store_true")
    ap.add_argument("--tries", type=int, default=1, help="re-plans per planner limit before giving up")
    ap.add_argument("--timeouts", type=float, nargs="+", default=[1.0], help="planner limits to try, seconds")
    args = ap.parse_args()
    with gzip.open(BATCH, "rt") as f:
        doc = json.load(f)
    items = doc["instances"]
    # failed re-plans and zero-valued prefixes are done again
    done = {i: r for i, r in load_progress(args.progress).items() if "error" not in r and r["float64"] != 0.0}
    if args.merge:
        n = 0
        for it in items:
            rec = done.get(it["index"])
            if rec and "float64" in rec:
                it["reference_prefix"] = {"slices": rec["slices"], "float64": rec["float64"]}
                if rec["slices"] == rec["of"] and it["reference_float64"] is None:
                    it["reference_float64"] = rec["float64"]
                n += 1
        data = json.dumps(doc, separators=(",", ":")).encode()
        with open(BATCH, "wb") as f:
            f.write(gzip.compress(data, mtime=0))
        print("merged", n, "prefix counts into", BATCH)
        return
    todo = [it for it in items if it["reference_float64"] is None and it["index"] not in done]
    # cost of one slice: per-slice work plus the slice-invariant part the reference recomputes
    todo.sort(key=lambda it: it["executed_flops"] / (1 << it["slice_groups"]))
    os.makedirs(os.path.dirname(args.progress), exist_ok=True)
    t0 = time.time()
    for k, it in enumerate(todo):
        rec = pin(it, args.tries, args.timeouts)
        with open(args.progress, "a") as f:
            f.write(json.dumps(rec) + "\n")
        print("%d/%d index %d %s %.0f s" % (k + 1, len(todo), it["index"], rec.get("error", "ok"),
                                             time.time() - t0), flush=True)


if __name__ == "__main__":
    main()
