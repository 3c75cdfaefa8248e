"""Cost models of a contraction plan, and candidate slice sets.

Three pieces:

* :func:`reference_estimate` restates the reference's planning-time cost model
  ``ContractionTreeContext.estimate_cost``
  (``contraction_methods/contraction_tree.pyx:382-496``): the memory cap of a
  post-order contraction in tensor entries (each join holds its result, and
  both operands twice for the transposes ``np.tensordot`` makes), the FLOP count
  ``sum 2^(log_terms + log_sums)`` -- which counts sliced edges as if unsliced
  (``:448-458``) -- the largest tensor rank and the best edge to slice next.
* :func:`join_table` and :func:`executed_cost` give the work this backend
  actually performs: GEMM extents over unsliced axes, joins that read no
  sliced edge run once per count (slice-invariant), the rest once per slice.
* :func:`greedy_slice_sequence` / :func:`slice_candidates` produce the slice
  sets a selector chooses among: classes of equivalent edges (edges joined
  through variable tensors, the closures of ``TensorNetwork.find_equivalent_edges``,
  ``tensor_network/tensor_network.pyx:470-489``) added one at a time by the
  reference's greedy memory rule (``slicers.py:27-33`` via ``best_edge``).
  Every slice set gives the same count: slicing a group only splits the sum
  over its shared value.

:func:`flop_model_seconds` is the plain FLOP/memory model a learned selector
falls back to: each join costs the larger of its FLOPs over a compute peak and
its bytes over a bandwidth peak.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, Iterable, List, Optional, Sequence, Set

from .program import Program, join_edges


@dataclass
class JoinShape:
    """One join over unsliced axes: log2 extents of the GEMM it is."""

    index: int          # post-order join index
    lm: int             # log2 M: left free axes
    ln: int             # log2 N: right free axes
    lk: int             # log2 K: shared axes
    per_slice: bool     # False when the join's subtree reads no sliced edge
    left_leaf: bool
    right_leaf: bool

    @property
    def flops(self) -> float:
        return 2.0 * 2.0 ** (self.lm + self.ln + self.lk)

    def bytes(self, elem: int) -> float:
        return elem * (2.0 ** (self.lm + self.lk) + 2.0 ** (self.ln + self.lk) + 2.0 ** (self.lm + self.ln))


def join_table(program: Program) -> List[JoinShape]:
    """Per join in post-order, mirroring the backend's lowering (the root is
    always counted per slice, and an unsliced program has no invariant joins)."""
    sliced = {e for g in program.slice_groups for e in g}
    stack = []  # (unsliced edges, depends on a sliced edge, is leaf)
    out: List[JoinShape] = []
    for t in program.postorder:
        if t >= 0:
            axes = program.leaves[t].axes
            stack.append(([e for e in axes if e not in sliced], any(e in sliced for e in axes), True))
        else:
            r, rdep, rleaf = stack.pop()
            l, ldep, lleaf = stack.pop()
            lmap, _, free = join_edges(l, r)
            k = len(lmap)
            out.append(JoinShape(len(out), len(l) - k, len(r) - k, k, ldep or rdep, lleaf, rleaf))
            stack.append((free, ldep or rdep, False))
    if out:
        out[-1].per_slice = True
    if not program.slice_groups:
        for j in out:
            j.per_slice = True
    return out


def executed_cost(program: Program, elem: int = 4) -> Dict[str, float]:
    """FLOPs and algorithmic bytes of one complete count as this backend runs
    it, next to the reference's per-slice work times the slice count."""
    S = program.num_slices
    js = join_table(program)
    per_f = sum(j.flops for j in js if j.per_slice)
    once_f = sum(j.flops for j in js if not j.per_slice)
    per_b = sum(j.bytes(elem) for j in js if j.per_slice)
    once_b = sum(j.bytes(elem) for j in js if not j.per_slice)
    return {"slices": S, "flops": per_f * S + once_f, "bytes": per_b * S + once_b,
            "flops_reference_order": (per_f + once_f) * S, "max_rank": max_rank(program)}


def max_rank(program: Program) -> int:
    sliced = {e for g in program.slice_groups for e in g}
    best = max((len([e for e in l.axes if e not in sliced]) for l in program.leaves), default=0)
    stack = []
    for t in program.postorder:
        if t >= 0:
            stack.append([e for e in program.leaves[t].axes if e not in sliced])
        else:
            r = stack.pop()
            l = stack.pop()
            _, _, free = join_edges(l, r)
            best = max(best, len(free))
            stack.append(free)
    return best


@dataclass
class CostInfo:
    flops: float
    total_memory: float
    local_memory: float
    largest_tensor: int
    best_edge: int
    best_edge_memory: float
    open_edge_total_memory: Dict[int, float]
    free: List[int]


def reference_estimate(program: Program, sliced_edges: Optional[Iterable[int]] = None) -> CostInfo:
    """The reference's ``estimate_cost`` from the root of the program's tree.

    ``sliced_edges`` defaults to the program's own slice groups.  Memory
    figures are in tensor entries; FLOPs use the reference's rule, which does
    not remove sliced edges."""
    sliced: Set[int] = set(sliced_edges) if sliced_edges is not None else {e for g in program.slice_groups for e in g}
    stack: List[CostInfo] = []
    for t in program.postorder:
        if t >= 0:
            free = list(program.leaves[t].axes)
            local = 2.0 ** sum(1 for e in free if e not in sliced)
            open_mem = {e: local / 2 for e in free if e not in sliced}
            stack.append(CostInfo(0.0, local, local, len(open_mem), -1, float(2 ** 64), open_mem, free))
            continue
        right = stack.pop()
        left = stack.pop()
        _, _, free = join_edges(left.free, right.free)
        local = 2.0 ** sum(1 for e in free if e not in sliced)
        left_cap = left.total_memory
        right_cap = left.local_memory + right.total_memory
        local_cap = local + 2 * left.local_memory + 2 * right.local_memory
        if left_cap >= right_cap and left_cap >= local_cap:
            total, best, best_mem = left_cap, left.best_edge, left.best_edge_memory
        elif right_cap >= local_cap:
            total, best, best_mem = right_cap, right.best_edge, left.local_memory + right.best_edge_memory
        else:
            total, best, best_mem = local_cap, left.best_edge, local_cap
        log_terms = (len(left.free) + len(right.free) - len(free)) // 2
        log_sums = len(free)
        flops = float(2 ** 100) if log_terms + log_sums > 100 else \
            left.flops + right.flops + float(2 ** (log_terms + log_sums))
        largest = max(sum(1 for e in free if e not in sliced), left.largest_tensor, right.largest_tensor)
        open_mem: Dict[int, float] = {}
        for e in left.free:
            if e not in right.open_edge_total_memory:
                open_mem[e] = max(left.open_edge_total_memory.get(e, 0.0),
                                  left.local_memory / 2 + right.total_memory,
                                  local / 2 + 2 * (left.local_memory / 2) + 2 * right.local_memory)
        for e in right.free:
            if e not in left.open_edge_total_memory:
                open_mem[e] = max(left.total_memory, left.local_memory + right.open_edge_total_memory.get(e, 0.0),
                                  local / 2 + 2 * left.local_memory + 2 * right.local_memory)
            elif e not in sliced:
                new_cap = max(left.open_edge_total_memory[e],
                              left.local_memory / 2 + right.open_edge_total_memory.get(e, 0.0),
                              local + 2 * (left.local_memory / 2) + 2 * (right.local_memory / 2))
                if new_cap < best_mem:
                    best, best_mem = e, new_cap
        stack.append(CostInfo(flops, total, local, largest, best, best_mem, open_mem, free))
    return stack[0]


def variable_groups(program: Program) -> Dict[int, List[int]]:
    """Edge -> its class of equivalent edges: the edges connected through
    variable (COPY) tensors, transitively, as ``find_equivalent_edges`` closes
    them; an edge on no variable tensor is its own class."""
    parent: Dict[int, int] = {}

    def find(x):
        while parent.setdefault(x, x) != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for leaf in program.leaves:
        for e in leaf.axes:
            find(e)
        if leaf.kind == "var":
            for e in leaf.axes[1:]:
                ra, rb = find(leaf.axes[0]), find(e)
                if ra != rb:
                    parent[rb] = ra
    classes: Dict[int, List[int]] = {}
    for e in list(parent):
        classes.setdefault(find(e), []).append(e)
    return {e: sorted(classes[find(e)]) for e in parent}


def with_groups(program: Program, groups: Sequence[Sequence[int]]) -> Program:
    """The same tree and leaves sliced by ``groups`` (replacing its own)."""
    return Program(program.leaves, program.postorder, [sorted(g) for g in groups], dict(program.meta)).validate()


def greedy_slice_sequence(program: Program, max_groups: int = 24) -> List[List[int]]:
    """Groups in the order the reference's greedy memory slicer adds them:
    repeatedly slice the group of the estimate's best edge, starting from the
    program's own slice groups."""
    groups = [sorted(g) for g in program.slice_groups]
    seq = list(groups)
    eq = variable_groups(program)
    sliced = {e for g in groups for e in g}
    while len(seq) < max_groups:
        info = reference_estimate(program, sliced)
        e = info.best_edge
        if e < 0 or e in sliced:
            break
        g = eq.get(e, [e])
        seq.append(g)
        sliced.update(g)
    return seq


def slice_candidates(program: Program, min_groups: int = 0, max_groups: int = 14) -> List[Program]:
    """Candidate slice sets: the first ``k`` groups of the greedy sequence for
    every ``k`` in ``[min_groups, max_groups]`` (fewer if the sequence ends)."""
    seq = greedy_slice_sequence(Program(program.leaves, program.postorder, []), max_groups)
    out = []
    for k in range(min_groups, min(max_groups, len(seq)) + 1):
        out.append(with_groups(program, seq[:k]))
    return out


def flop_model_seconds(program: Program, flops_per_s: float, bytes_per_s: float, elem: int = 4,
                       launch_s: float = 3e-6, slices_per_launch: Optional[int] = None) -> float:
    """Plain FLOP/memory model of one count: every join costs
    ``max(flops / flops_per_s, bytes / bytes_per_s)`` per run, per-slice joins
    run once per slice, and each launch of a chunk costs ``launch_s``."""
    S = program.num_slices
    B = S if slices_per_launch is None else max(1, min(S, slices_per_launch))
    chunks = (S + B - 1) // B
    t = 0.0
    for j in join_table(program):
        runs = S if j.per_slice else 1
        t += runs * max(j.flops / flops_per_s, j.bytes(elem) / bytes_per_s)
        t += (chunks if j.per_slice else 1) * launch_s
    return t
