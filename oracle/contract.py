"""CPU oracle for the contraction hot path -- TEST INFRASTRUCTURE ONLY.

Restates, in numpy FP64, the reference's execution of a sliced plan:

* ``contract_sliced``  -- ``tensor_apis/base_api.py:17-28``: for each slice in
  ``itertools.product`` order (``tensor_network.pyx:396-401``), contract the
  network and add ``result[()]`` into a plain FP64 running sum; an optional
  ``num_slice_limit`` keeps a prefix (``base_api.py:23-24``).
* ``contract``         -- ``TensorNetwork.identify`` (``tensor_network.pyx:142-156``):
  post-order stack machine; a leaf pushes its built tensor, a join pops right
  then left and pushes ``np.tensordot(left, right, (lmap, rmap))``
  (``numpy_apis.py:42-43``).
* leaf slicing     -- ``SlicedTensor.build`` (``tensor.py:66-68``) indexes the
  parent at the slice value and keeps a size-1 axis; this restatement drops the
  sliced axes instead (the values are identical) and removes them from the
  join's edge lists, as ``remove_sliced_indices_from``
  (``tensor_network.pyx:444-468``) does.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may use this module, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import numpy as np

from tensororder_gb300.program import Program, join_edges


def slice_values(program: Program, s: int):
    """Edge -> fixed value for slice ``s`` (last group varies fastest)."""
    G = len(program.slice_groups)
    fixed = {}
    for g, group in enumerate(program.slice_groups):
        v = (s >> (G - 1 - g)) & 1
        for e in group:
            fixed[e] = v
    return fixed


def build_leaf(leaf, fixed):
    """Leaf values for one slice with the sliced axes removed; returns
    ``(array, remaining_edges)``."""
    parent = leaf.parent()
    index = []
    edges = []
    for e in leaf.axes:
        if e in fixed:
            index.append(fixed[e])
        else:
            index.append(slice(0, 2))
            edges.append(e)
    return parent[tuple(index)], edges


def contract(program: Program, s: int = 0, dtype=np.float64):
    """Contract slice ``s``; returns the root tensor (a 0-d array for CNF
    networks) and its edge list."""
    fixed = slice_values(program, s)
    stack = []
    for t in program.postorder:
        if t >= 0:
            arr, edges = build_leaf(program.leaves[t], fixed)
            stack.append((arr.astype(dtype, copy=False), edges))
        else:
            right, redges = stack.pop()
            left, ledges = stack.pop()
            lmap, rmap, free = join_edges(ledges, redges)
            stack.append((np.tensordot(left, right, (lmap, rmap)), free))
    return stack[0]


def contract_sliced(program: Program, num_slice_limit=None, dtype=np.float64):
    """Sum of all slice contractions with a plain running sum, as
    ``base_api.py:21-28`` does."""
    n = program.num_slices
    if num_slice_limit is not None:
        n = min(n, int(num_slice_limit))
    result = 0
    for s in range(n):
        arr, _ = contract(program, s, dtype)
        result += arr[()]
    return result


def join_shapes(program: Program):
    """Per-join ``(M, N, K)`` over unsliced axes, in post-order (one slice).

    M = 2^(left free), N = 2^(right free), K = 2^(shared): the GEMM that
    ``np.tensordot`` hands to BLAS.
    """
    sliced = {e for g in program.slice_groups for e in g}
    stack = []
    out = []
    for t in program.postorder:
        if t >= 0:
            stack.append([e for e in program.leaves[t].axes if e not in sliced])
        else:
            r = stack.pop()
            l = stack.pop()
            lmap, rmap, free = join_edges(l, r)
            k = len(lmap)
            out.append((1 << (len(l) - k), 1 << (len(r) - k), 1 << k))
            stack.append(free)
    return out


def algorithmic_flops(program: Program, num_slices=None):
    """Sum over joins of 2*M*N*K, times the number of slices."""
    per_slice = sum(2 * m * n * k for m, n, k in join_shapes(program))
    return per_slice * (program.num_slices if num_slices is None else num_slices)
