"""The plugin's program cache, on the host (no GPU).

``GB300API`` keeps its last device program, keyed by what the lowering depends
on: the tree, the slice groups and every leaf's axes and kind.  A count of the
same network with other weights uploads the new leaves into that program
(``set_leaves``); any other network releases it and lowers a new one.  A stand-in
device program records the calls.
"""
import copy

import numpy as np
import pytest

from tensororder_gb300 import api, runtime
from tensororder_gb300.program import Leaf, Program


class FakeInfo:
    flops_per_slice = 1e6
    root_rank = 0


class FakeDeviceProgram:
    made = []

    def __init__(self, program, device=0):
        self.info = FakeInfo()
        self.program = program
        self.uploads = []
        self.closed = False
        FakeDeviceProgram.made.append(self)

    def set_leaves(self, program, stream=None):
        self.uploads.append(program)
        self.program = program

    def close(self):
        self.closed = True

    def reset(self, stream=None):
        pass

    def allocate_workspace(self, mode, slices, max_fraction=0.5):
        return None

    def run(self, mode, begin=0, end=None, workspace=None, stream=None):
        pass

    def result(self, stream=None):
        # the "count": the sum of the variables' w_neg, so uploads are visible
        return np.array(sum(l.w_neg for l in self.program.leaves if l.kind == "var"))


@pytest.fixture
def backend(monkeypatch):
    FakeDeviceProgram.made = []
    monkeypatch.setattr(runtime, "DeviceProgram", FakeDeviceProgram)
    monkeypatch.setattr(api.GB300API, "_stream", lambda self: None)
    monkeypatch.setattr(api.GB300API, "_wait", staticmethod(lambda stream: None))
    return api.GB300SplitAPI()


def network(w=0.3, groups=2):
    leaves = [Leaf([0, 1], "or", positive=[True, False]), Leaf([0], "var", w_neg=w, w_pos=1 - w),
              Leaf([1], "var", w_neg=0.5, w_pos=0.5)]
    for i in range(groups):
        leaves.append(Leaf([2 + i], "var", w_neg=0.25, w_pos=0.75))
    tokens = [0, 1, -1, 2, -1]
    for i in range(groups):
        tokens += [3 + i, -1]
    return Program(leaves, tokens, [[2 + i] for i in range(groups)]).validate()


def test_same_structure_reuses_the_program_and_uploads_leaves(backend):
    p1, p2 = network(0.3), network(0.6)
    v1 = float(backend.contract_program(p1))
    v2 = float(backend.contract_program(p2))
    assert len(FakeDeviceProgram.made) == 1
    dp = FakeDeviceProgram.made[0]
    assert dp.uploads == [p2] and not dp.closed
    assert v1 == pytest.approx(0.3 + 0.5 + 0.25 + 0.25) and v2 == pytest.approx(0.6 + 0.5 + 0.25 + 0.25)


def test_other_structure_releases_the_cached_program(backend):
    backend.contract_program(network(groups=2))
    backend.contract_program(network(groups=3))  # another slice group: another lowering
    assert len(FakeDeviceProgram.made) == 2
    assert FakeDeviceProgram.made[0].closed and not FakeDeviceProgram.made[1].closed


@pytest.mark.parametrize("change", ["axes", "kind", "tree"])
def test_what_the_key_covers(change):
    p = network()
    q = copy.deepcopy(p)
    if change == "axes":
        q.leaves[1].axes = [1]
        q.leaves[2].axes = [0]
    elif change == "kind":
        q.leaves[1].kind, q.leaves[1].values = "dense", q.leaves[1].parent()
    else:
        q.postorder = [0, 2, -1, 1, -1] + q.postorder[5:]
    assert api.GB300API._structure_key(p) != api.GB300API._structure_key(q)
    # weights and clause polarities are not part of the key
    r = copy.deepcopy(p)
    r.leaves[1].w_neg = 0.9
    r.leaves[0].positive = [False, True]
    assert api.GB300API._structure_key(p) == api.GB300API._structure_key(r)


def test_cache_can_be_switched_off(backend):
    backend.cache_programs = False
    backend.contract_program(network(0.3))
    backend.contract_program(network(0.6))
    assert len(FakeDeviceProgram.made) == 2
    assert all(not dp.uploads for dp in FakeDeviceProgram.made)
