"""Join programs: the flat form of a TensorOrder ``SlicedExecutionPlan``.

A plan in the reference is three Python objects: a ``ContractionTree``
(``contraction_methods/contraction_tree.pyx:4-183``), a ``TensorNetwork``
(``tensor_network/tensor_network.pyx:11-502``) and ``groups_to_slice``
(``tensor_network/sliced_execution_plan.py:19-20``).  Execution walks the tree
in post-order (``tensor_network.pyx:142-156``), building each leaf and joining
the top two stack entries with ``tensordot``; the slice loop
(``tensor_apis/base_api.py:17-28``) repeats that for every assignment of the
sliced edge groups.

A :class:`Program` keeps exactly what that walk needs:

* ``leaves``   -- one entry per tensor in post-order of the tree: its edge ids
  (the tensor's ``index_list`` order, which is the axis order of the tensor
  ``Tensor.build`` returns) and its values, either as a compact descriptor of
  the two CNF tensor kinds (``tensor_network_constructions.py:69-152``) or as
  a dense row-major array;
* ``postorder`` -- the post-order token stream: ``i >= 0`` pushes leaf ``i``,
  ``-1`` pops right then left and pushes their join;
* ``slice_groups`` -- the non-empty edge groups of ``groups_to_slice`` in plan
  order.  Slice ``s`` (0-based, in ``itertools.product`` order as
  ``tensor_network.pyx:396-401`` enumerates it) fixes every edge of group
  ``g`` to bit ``G-1-g`` of ``s``.

Every index has dimension 2 (binary CNF tensors); anything else is rejected.
The file format is JSON (``to_json``/``from_json``); float weights round-trip
exactly through ``repr``.
"""
from __future__ import annotations

import gzip
import json
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

FORMAT = "togb.program/1"


@dataclass
class Leaf:
    axes: List[int]
    kind: str  # "or" | "var" | "dense"
    positive: Optional[List[bool]] = None  # "or": literal polarity per axis
    output_index: Optional[int] = None  # "or": factored OR gate output axis
    w_neg: float = 1.0  # "var": value at the all-0 corner
    w_pos: float = 1.0  # "var": value at the all-1 corner
    values: Optional[np.ndarray] = None  # "dense": shape (2,)*rank, float64

    @property
    def rank(self) -> int:
        return len(self.axes)

    def parent(self) -> np.ndarray:
        """Dense float64 values of the unsliced tensor, shape ``(2,)*rank``.

        Restates ``OrTensor.build`` (``tensor_network_constructions.py:69-99``)
        and ``VariableTensor.build`` (``tensor_network_constructions.py:144-152``).
        """
        r = self.rank
        if self.kind == "dense":
            return np.asarray(self.values, dtype=np.float64).reshape((2,) * r)
        if self.kind == "var":
            out = np.zeros((2,) * r, dtype=np.float64)
            if r == 0:
                out[()] = self.w_neg + self.w_pos
            else:
                out[(0,) * r] = self.w_neg
                out[(1,) * r] = self.w_pos
            return out
        if self.kind == "or":
            out = np.ones((2,) * r, dtype=np.float64)
            all_false = [0 if p else 1 for p in self.positive]
            if self.output_index is None:
                out[tuple(all_false)] = 0
            else:
                o = self.output_index
                o_false = 0 if self.positive[o] else 1
                out[tuple(o_false if i == o else slice(0, 2) for i in range(r))] = 0
                out[tuple(all_false)] = 1
                all_false[o] = 1 - all_false[o]
                out[tuple(all_false)] = 0
            return out
        raise ValueError("unknown leaf kind %r" % self.kind)

    def to_dict(self):
        d = {"axes": [int(a) for a in self.axes], "kind": self.kind}
        if self.kind == "or":
            d["positive"] = [bool(p) for p in self.positive]
            if self.output_index is not None:
                d["output_index"] = int(self.output_index)
        elif self.kind == "var":
            d["w"] = [float(self.w_neg), float(self.w_pos)]
        else:
            d["values"] = [float(v) for v in np.asarray(self.values, dtype=np.float64).ravel()]
        return d

    @staticmethod
    def from_dict(d):
        kind = d["kind"]
        if kind == "or":
            return Leaf(list(d["axes"]), "or", positive=list(d["positive"]),
                        output_index=d.get("output_index"))
        if kind == "var":
            return Leaf(list(d["axes"]), "var", w_neg=float(d["w"][0]), w_pos=float(d["w"][1]))
        if kind == "dense":
            r = len(d["axes"])
            return Leaf(list(d["axes"]), "dense",
                        values=np.asarray(d["values"], dtype=np.float64).reshape((2,) * r))
        raise ValueError("unknown leaf kind %r" % kind)


@dataclass
class Program:
    leaves: List[Leaf]
    postorder: List[int]
    slice_groups: List[List[int]] = field(default_factory=list)
    meta: dict = field(default_factory=dict)

    @property
    def num_slices(self) -> int:
        return 1 << len(self.slice_groups)

    @property
    def num_joins(self) -> int:
        return sum(1 for t in self.postorder if t < 0)

    def validate(self):
        depth = 0
        seen = set()
        for t in self.postorder:
            if t >= 0:
                if t in seen or t >= len(self.leaves):
                    raise ValueError("leaf %d pushed twice or out of range" % t)
                seen.add(t)
                depth += 1
            else:
                if depth < 2:
                    raise ValueError("join with fewer than two operands on the stack")
                depth -= 1
        if depth != 1 or len(seen) != len(self.leaves):
            raise ValueError("post-order does not reduce to a single tensor")
        sliced = set()
        for g in self.slice_groups:
            if not g:
                raise ValueError("empty slice group")
            for e in g:
                if e in sliced:
                    raise ValueError("edge %d in two slice groups" % e)
                sliced.add(e)
        return self

    def to_dict(self):
        return {
            "format": FORMAT,
            "leaves": [l.to_dict() for l in self.leaves],
            "postorder": [int(t) for t in self.postorder],
            "slice_groups": [sorted(int(e) for e in g) for g in self.slice_groups],
            "meta": self.meta,
        }

    @staticmethod
    def from_dict(d):
        if d.get("format") != FORMAT:
            raise ValueError("not a %s document" % FORMAT)
        return Program(
            leaves=[Leaf.from_dict(x) for x in d["leaves"]],
            postorder=list(d["postorder"]),
            slice_groups=[list(g) for g in d["slice_groups"]],
            meta=dict(d.get("meta", {})),
        ).validate()

    def dump(self, path):
        data = json.dumps(self.to_dict(), separators=(",", ":")).encode()
        if str(path).endswith(".gz"):
            data = gzip.compress(data, mtime=0)
        with open(path, "wb") as f:
            f.write(data)

    @staticmethod
    def load(path):
        with open(path, "rb") as f:
            data = f.read()
        if str(path).endswith(".gz"):
            data = gzip.decompress(data)
        return Program.from_dict(json.loads(data))


def _leaf_from_reference_tensor(tensor, axes):
    """Describe one reference leaf.  OR/variable tensors keep their compact
    parameters; everything else (``BuiltTensor`` from ``--early``, factored
    tensors) is materialised with the tensor's own ``build``."""
    if len(tensor.shape) != len(axes):
        raise ValueError("tensor rank and index list disagree")
    if any(int(d) not in (1, 2) for d in tensor.shape):
        raise ValueError("only binary (dimension-2) indices are supported")
    name = type(tensor).__name__
    if any(int(d) == 1 for d in tensor.shape):
        name = "sliced"
    if name == "OrTensor":
        return Leaf(list(axes), "or", positive=[bool(p) for p in tensor._OrTensor__literals_positive],
                    output_index=tensor._OrTensor__output_index)
    if name == "VariableTensor":
        return Leaf(list(axes), "var", w_neg=float(tensor._VariableTensor__negative_weight),
                    w_pos=float(tensor._VariableTensor__positive_weight))

    def factory(shape, default_value=None):
        if default_value is None:
            return np.empty(shape, dtype=np.float64)
        return np.full(shape, default_value, dtype=np.float64)

    values = np.asarray(tensor.build(factory), dtype=np.float64)
    if any(d == 1 for d in values.shape):
        # A network already sliced by slice_groups keeps each sliced axis with
        # size 1 (tensor.py:66-68).  Both endpoints of such an edge are padded
        # to size 2 with zeros at index 1: the contraction over the edge gains
        # only 0*0 terms, so the value is unchanged.
        padded = np.zeros((2,) * values.ndim, dtype=np.float64)
        padded[tuple(slice(0, d) for d in values.shape)] = values
        values = padded
    return Leaf(list(axes), "dense", values=values.reshape((2,) * len(axes)))


def from_plan(plan) -> Program:
    """Flatten a reference ``SlicedExecutionPlan`` (duck-typed: ``plan.tree``,
    ``plan.network``, ``plan.groups_to_slice``).

    The walk mirrors ``TensorNetwork.identify`` (``tensor_network.pyx:142-156``).
    Each join's edge maps are re-derived from the operands' edge lists by the
    rule of ``compute_join_properties`` (``contraction_tree.pyx:248-288``) and
    checked against the tree's own ``left_edge_map``/``right_edge_map``.
    """
    network = plan.network
    leaves: List[Leaf] = []
    postorder: List[int] = []
    stack: List[List[int]] = []
    for node in plan.tree.iterate_postorder():
        if node.is_leaf:
            tid = node.tensor_index
            axes = [int(e) for e in network.index_list(tid)]
            leaves.append(_leaf_from_reference_tensor(network[tid], axes))
            postorder.append(len(leaves) - 1)
            stack.append(axes)
        else:
            right = stack.pop()
            left = stack.pop()
            lmap, rmap, free = join_edges(left, right)
            if list(node.left_edge_map) != lmap or list(node.right_edge_map) != rmap:
                raise ValueError("tree edge maps disagree with the operands' edge lists")
            postorder.append(-1)
            stack.append(free)
    groups = [sorted(int(e) for e in g) for g in plan.groups_to_slice if len(g) > 0]
    return Program(leaves, postorder, groups).validate()


def join_edges(left, right):
    """Shared-edge positions and output edge order of one join, by the rule of
    ``compute_join_properties`` (``contraction_tree.pyx:264-282``): a left edge
    found in the right list is shared (paired with its first match); the output
    is the unshared left edges in order, then the unshared right edges in order
    -- the same axis order ``np.tensordot`` produces."""
    lmap, rmap, free = [], [], []
    for i, e in enumerate(left):
        j = next((j for j, f in enumerate(right) if f == e), None)
        if j is None:
            free.append(e)
        else:
            lmap.append(i)
            rmap.append(j)
    lset = set(left)
    free.extend(e for e in right if e not in lset)
    return lmap, rmap, free
