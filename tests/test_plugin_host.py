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
    h = api.GB300API()
    h.add_argument("entry_type", "float16")  # FP32 storage: at least float16
    assert h._mode == runtime.MODE_SPLIT and h.get_entry_size() == 4
    for name, word in (("int", np.int64), ("uint", np.uint64)):
        q = api.GB300SplitAPI()
        q.add_argument("entry_type", name)
        assert q._mode == runtime.MODE_INT64 and q._word_type is word and q.get_entry_size() == 8
    b = api.GB300SplitAPI()
    b.add_argument("entry_type", "bigint")  # exact integers through the int forms
    assert b._bigint and b.get_entry_size() == 8
    b.add_argument("entry_type", "float32")
    assert not b._bigint and b.get_entry_size() == 4
    with pytest.raises(ValueError):
        p.add_argument("entry_type", "complex128")
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


def _device_leaf_formula(spec, rank):
    """The value rule of the library's leaf-building kernel (k_build_leaves),
    restated on the host from a togb_leaf_spec."""
    n = 1 << rank
    out = np.zeros(n)
    if spec.kind == runtime.LEAF_VARIABLE:
        if rank == 0:
            return np.array(spec.w_neg + spec.w_pos)
        out[0], out[n - 1] = spec.w_neg, spec.w_pos
        return out.reshape((2,) * rank)
    F = sum(1 << (rank - 1 - a) for a in range(rank) if not (spec.positive >> a) & 1)
    for i in range(n):
        if spec.output_index < 0:
            out[i] = 0.0 if i == F else 1.0
        else:
            bo = 1 << (rank - 1 - spec.output_index)
            out[i] = 1.0 if i == F else (0.0 if i == (F ^ bo) else (1.0 if (i ^ F) & bo else 0.0))
    return out.reshape((2,) * rank)


@pytest.mark.parametrize("name", golden_names())
def test_leaf_specs_describe_the_reference_leaves(name):
    """Every clause and variable leaf, encoded as togb_leaf_spec, expands by the
    device kernel's rule to the values OrTensor/VariableTensor.build give."""
    prog = Program.from_dict(load_golden(name)["program"])
    d = runtime._Desc(prog, values="dense")
    for i, leaf in enumerate(prog.leaves):
        spec = d.specs[i]
        if spec.kind == runtime.LEAF_DENSE:
            assert leaf.kind == "dense"
            continue
        assert np.array_equal(_device_leaf_formula(spec, leaf.rank), leaf.parent())
