"""Host-side behaviour of the --tensor_library plugin that needs no GPU:
argument handling (numpy_apis.py:13-34, base_api.py:9-12), entry sizes,
registration into ALL_APIS, and plan flattening of duck-typed plans."""
import sys
import types

import numpy as np
import pytest

from conftest import golden_names, load_golden
from fakeplan import FakePlan
from tensororder_gb300 import api, runtime
from tensororder_gb300.program import Program, from_plan


def test_entry_types_and_sizes():
    p = api.GB300API()
    p.add_argument("entry_type", "float64")
    assert p.get_entry_size() == 8
    p.add_argument("entry_type", "float32")
    assert p.get_entry_size() == 4
    s = api.GB300SplitAPI()
    s.add_argument("entry_type", "float64")
    assert s.get_entry_size() == 4
    with pytest.raises(ValueError):
        p.add_argument("entry_type", "float16")
    with pytest.raises(ValueError):
        p.add_argument("tpu", "1.2.3.4")
    p.add_argument("thread_limit", 1)


def test_create_tensor_matches_numpy_factory():
    p = api.GB300API()
    assert p.create_tensor((2, 2), 1).dtype == np.float64
    assert np.all(p.create_tensor((2, 2, 2), 0) == 0)


def test_register_into_reference_registry(monkeypatch):
    class OOM(Exception):
        pass

    fake = types.ModuleType("tensor_network")
    fake.ALL_APIS = {"numpy": object}
    fake.OutOfMemoryError = OOM
    monkeypatch.setitem(sys.modules, "tensor_network", fake)
    monkeypatch.setattr(api, "_OOM", api._OOM)  # restored after the test
    reg = api.register()
    assert reg["gb300"] is api.GB300API and reg["gb300-split"] is api.GB300SplitAPI
    assert "numpy" in reg
    assert api._OOM is OOM


@pytest.mark.parametrize("name", golden_names())
def test_from_plan_round_trips_duck_typed_plans(name):
    prog = Program.from_dict(load_golden(name)["program"])
    again = from_plan(FakePlan(prog))
    assert again.postorder == prog.postorder
    assert again.slice_groups == [sorted(g) for g in prog.slice_groups]
    for a, b in zip(prog.leaves, again.leaves):
        assert a.axes == b.axes
        assert np.array_equal(a.parent(), b.parent())


def test_from_plan_rejects_mismatched_edge_maps():
    prog = Program.from_dict(load_golden("wvc18_s2")["program"])
    plan = FakePlan(prog)
    for node in plan.tree._nodes:
        if not node.is_leaf and node.left_edge_map:
            node.left_edge_map = list(reversed(node.left_edge_map)) + [99]
            break
    with pytest.raises(ValueError):
        from_plan(plan)


def test_oom_maps_to_reference_error(monkeypatch):
    class Boom(runtime.DeviceProgram):
        def __init__(self, *a, **k):
            raise runtime.DeviceOutOfMemory(runtime.ERR_OOM, "forced")

    monkeypatch.setattr(runtime, "DeviceProgram", Boom)
    monkeypatch.setitem(sys.modules, "torch", types.SimpleNamespace(cuda=types.SimpleNamespace(
        current_stream=lambda *a: None)))
    prog = Program.from_dict(load_golden("wvc18_s2")["program"])
    with pytest.raises(api._OOM):
        api.GB300API().contract_program(prog)
