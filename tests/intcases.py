"""Cases for the int form (64-bit words, sums and products modulo 2^64).

The reference's ``int`` and ``uint`` entry types contract numpy int64 / uint64
tensors (``numpy_apis.py:15-22``), whose arithmetic wraps modulo 2^64.  Every
summation order gives the same words there, so the int form must equal the
oracle in int64 bit for bit, whatever kernels and slice chunks run.
"""
import copy

import numpy as np

from oracle import contract as oracle
from tensororder_gb300.program import join_edges

MOD = 1 << 64


def integer_weights(prog, w_neg=3, w_pos=5):
    """The same network with integer variable weights (stored as floats, as
    the reference's weights are) and dense leaves (partial contractions)
    scaled by 8 and rounded up (zeros stay zeros): every leaf value an
    integer, counts far beyond 2^64, so every join and the slice sum wrap."""
    out = copy.deepcopy(prog)
    for l in out.leaves:
        if l.kind == "var":
            l.w_neg, l.w_pos = float(w_neg), float(w_pos)
        elif l.kind == "dense":
            l.values = np.ceil(np.asarray(l.values, dtype=np.float64) * 8.0)
    return out


def exact_count(prog, begin=0, end=None):
    """The count in Python integers (no wrap) over slices [begin, end): leaves
    converted toward zero as numpy's float-to-int64 cast does, then contracted
    as object arrays."""
    total = 0
    for s in range(begin, prog.num_slices if end is None else end):
        fixed = oracle.slice_values(prog, s)
        stack = []
        for t in prog.postorder:
            if t >= 0:
                arr, edges = oracle.build_leaf(prog.leaves[t], fixed)
                stack.append((arr.astype(np.int64).astype(object), edges))
            else:
                right, redges = stack.pop()
                left, ledges = stack.pop()
                lmap, rmap, free = join_edges(ledges, redges)
                stack.append((np.tensordot(left, right, (lmap, rmap)), free))
        total += int(np.asarray(stack[0][0]).reshape(-1)[0])
    return total


def oracle_words(prog, num_slice_limit=None):
    """The oracle's int64 count as a uint64 word (the sum modulo 2^64)."""
    with np.errstate(over="ignore"):
        v = oracle.contract_sliced(prog, num_slice_limit, dtype=np.int64)
    return np.int64(v).view(np.uint64)
