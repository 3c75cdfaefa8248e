"""Pairwise-contraction sweep on the GPU: plain FP64 against the split form.

    python -m tensororder_gb300.run_sweep [--shapes a,b,k ...] [--slices S]

Each case contracts two seeded dense tensors X (rank a) and Y (rank b), all
index dimensions 2, entries uniform in [0.5, 1.5], sharing k indices at random
axis positions; X and Y are themselves built on the device as outer products
of two leaves each, so the measured join is a join of two intermediates (the
shape GEMM joins take inside plans).  ``--slices S`` adds log2(S) slice groups
on Y's leaves, so the join runs over S slices in one launch.  For every case
and form it reports the join's device time (CUDA events), TFLOP/s
(2*M*N*K per slice), the kernel the library chose, and the relative error of
the result against ``np.tensordot`` in FP64 (the reference's contraction,
``numpy_apis.py:42-43``), computed on the host from the same inputs.  Cases too
large for a full host contraction (M*N*K*slices > 2^36) are checked on a seeded
sample of 4096 output entries, each an explicit K-long FP64 dot product of the
operands' fibres (:func:`sampled_check`).
"""
from __future__ import annotations

import argparse
import json
import sys

import numpy as np

from . import runtime
from .program import Leaf, Program, join_edges

DEFAULT_SHAPES = [(10, 10, 5), (14, 14, 7), (16, 16, 8), (18, 18, 9), (20, 20, 10), (22, 22, 11), (24, 22, 12),
                  (24, 24, 12), (26, 24, 12), (26, 25, 14), (28, 28, 14), (12, 24, 4), (24, 12, 2), (20, 8, 0)]


def case(seed, a, b, k, slice_bits=0):
    rng = np.random.default_rng(seed)
    shared = list(range(k))
    fa = list(range(k, a))
    fb = list(range(a, a + b - k))
    x_axes = list(rng.permutation(fa + shared))
    y_axes = list(rng.permutation(shared + fb))
    leaves = []
    for axes in (x_axes, y_axes):
        cut = len(axes) // 2
        for h in (axes[:cut], axes[cut:]):
            leaves.append(Leaf([int(e) for e in h], "dense", values=rng.uniform(0.5, 1.5, size=(2,) * len(h))))
    groups = []
    base = a + b - k
    for g in range(slice_bits):
        e = base + g
        leaves[2].axes.append(e)
        leaves[3].axes.append(e)
        groups.append([e])
    if slice_bits:
        for l in leaves[2:]:
            l.values = rng.uniform(0.5, 1.5, size=(2,) * l.rank)
    return Program(leaves, [0, 1, -1, 2, 3, -1, -1], groups).validate()


def host_result(prog):
    """Sum over slices of np.tensordot of the two intermediates, FP64."""
    def build(i, j, fixed):
        out = []
        for li in (i, j):
            l = prog.leaves[li]
            idx = tuple(fixed.get(e, slice(None)) for e in l.axes)
            out.append((l.parent()[idx], [e for e in l.axes if e not in fixed]))
        (p, pe), (q, qe) = out
        lm, rm, free = join_edges(pe, qe)
        return np.tensordot(p, q, (lm, rm)), free

    G = len(prog.slice_groups)
    total = None
    for s in range(prog.num_slices):
        fixed = {g[0]: (s >> (G - 1 - n)) & 1 for n, g in enumerate(prog.slice_groups)}
        X, xe = build(0, 1, fixed)
        Y, ye = build(2, 3, fixed)
        lm, rm, _ = join_edges(xe, ye)
        r = np.tensordot(X, Y, (lm, rm))
        total = r if total is None else total + r
    return total


def operand_matrices(prog):
    """The two intermediates of an unsliced case as host FP64 matrices
    X2[m, k] and Y2[n, k]: rows over the free axes in the operand's own axis
    order (the order of the result's axes), columns over the shared axes in
    one common order.  Returns ``(X2, Y2)``."""
    if prog.slice_groups:
        raise ValueError("sampled checks cover unsliced cases")

    def operand(i, j):
        p, q = prog.leaves[i], prog.leaves[j]
        return np.multiply.outer(p.parent(), q.parent()), list(p.axes) + list(q.axes)

    X, xe = operand(0, 1)
    Y, ye = operand(2, 3)
    shared = sorted(set(xe) & set(ye))
    fx = [e for e in xe if e not in shared]
    fy = [e for e in ye if e not in shared]
    K = 1 << len(shared)
    X2 = X.transpose([xe.index(e) for e in fx + shared]).reshape(1 << len(fx), K)
    Y2 = Y.transpose([ye.index(e) for e in fy + shared]).reshape(1 << len(fy), K)
    return X2, Y2


def sampled_check(prog, result, samples=4096, seed=0):
    """Largest relative error of ``result`` (the device's root tensor in the
    reference's axis order) over ``samples`` seeded output entries, each
    recomputed on the host as sum_k X2[m, k] * Y2[n, k] in FP64."""
    X2, Y2 = operand_matrices(prog)
    M, N = X2.shape[0], Y2.shape[0]
    rng = np.random.default_rng(seed)
    ms = rng.integers(0, M, size=samples)
    ns = rng.integers(0, N, size=samples)
    want = np.einsum("ij,ij->i", X2[ms], Y2[ns])
    got = np.asarray(result).reshape(M, N)[ms, ns]
    return float(np.max(np.abs(got - want) / np.abs(want)))


def run_case(prog, mode, repeats=3):
    import torch

    dp = runtime.DeviceProgram(prog)
    ws = dp.allocate_workspace(mode, dp.num_slices, max_fraction=0.6)
    dp.set_timing(True)
    best = None
    for _ in range(repeats):
        dp.reset()
        dp.run(mode, workspace=ws)
        torch.cuda.synchronize()
        t = dp.join_times()[-1]
        best = t if best is None else min(best, t)
    res = dp.result()
    kern = int(dp.joins(mode)[-1][3])
    dp.close()
    return res, best, kern


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--shapes", nargs="*", default=None)
    ap.add_argument("--slices", type=int, default=1)
    ap.add_argument("--no-check", action="store_true", help="skip the host FP64 result (large cases)")
    args = ap.parse_args(argv)
    shapes = [tuple(int(x) for x in s.split(",")) for s in args.shapes] if args.shapes else DEFAULT_SHAPES
    sb = max(0, int(np.log2(max(1, args.slices))))
    for i, (a, b, k) in enumerate(shapes):
        if a + b - 2 * k > 30:
            continue
        prog = case(100 + i, a, b, k, sb)
        M, N, K = 2 ** (a - k), 2 ** (b - k), 2 ** k
        flops = 2.0 * M * N * K * prog.num_slices
        small = M * N * K * prog.num_slices <= 2 ** 36
        ref = None if args.no_check or not small else host_result(prog)
        sampled = not args.no_check and not small and not prog.slice_groups
        line = {"a": a, "b": b, "k": k, "M": M, "N": N, "K": K, "slices": prog.num_slices}
        for name, mode in (("plain_f64", runtime.MODE_F64), ("split", runtime.MODE_SPLIT)):
            res, ms, kern = run_case(prog, mode)
            entry = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "kernel": runtime.KERNEL_NAMES[kern]}
            if ref is not None:
                entry["max_rel_err"] = float(np.max(np.abs(res - ref)) / np.max(np.abs(ref)))
            elif sampled:
                entry["max_rel_err_sampled"] = sampled_check(prog, res)
            line[name] = entry
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
