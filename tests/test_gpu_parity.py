"""Parity of the CUDA path with the reference's own counts (golden vectors
made by running the reference's numpy backend on the same frozen plans).

Tolerances: plain FP64 form <= 1e-12 relative; split form <= 1e-6 relative."""
import gzip
import json
import os

import numpy as np
import pytest

from conftest import ROOT, golden_names, load_golden
from fakeplan import FakePlan
from tensororder_gb300 import api, runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu

NAMES = golden_names()
PLAIN_TOL = 1e-12
SPLIT_TOL = 1e-6


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def program(name):
    return Program.from_dict(load_golden(name)["program"])


@pytest.mark.parametrize("name", NAMES)
def test_plain_count_matches_reference(name, cuda):
    doc = load_golden(name)
    got = float(api.GB300API().contract_program(program(name)))
    assert rel(got, doc["reference"]["float64"]) <= PLAIN_TOL
    if "bigint" in doc["reference"] and int(doc["reference"]["bigint"]) < 2 ** 53:
        assert got == float(int(doc["reference"]["bigint"]))


@pytest.mark.parametrize("name", NAMES)
def test_split_count_matches_reference(name, cuda):
    doc = load_golden(name)
    got = float(api.GB300SplitAPI().contract_program(program(name)))
    assert rel(got, doc["reference"]["float64"]) <= SPLIT_TOL


@pytest.mark.parametrize("name", [n for n in NAMES if "prefix_float64" in load_golden(n)["reference"]])
@pytest.mark.parametrize("mode", [runtime.MODE_F64, runtime.MODE_SPLIT])
def test_slice_prefixes(name, mode, cuda):
    doc = load_golden(name)
    full = doc["reference"]["float64"]
    tol = PLAIN_TOL if mode == runtime.MODE_F64 else SPLIT_TOL
    backend = api.GB300API(mode=mode)
    for k, want in enumerate(doc["reference"]["prefix_float64"], start=1):
        got = float(backend.contract_program(program(name), num_slice_limit=k))
        assert abs(got - want) <= tol * abs(full)


@pytest.mark.parametrize("mode", [runtime.MODE_F64, runtime.MODE_SPLIT])
@pytest.mark.parametrize("chunk", [1, 3, 5])
def test_chunked_workspace_gives_same_count(mode, chunk, cuda):
    import torch

    prog = program("vc60_s4")
    dp = runtime.DeviceProgram(prog)
    ws = torch.empty(dp.workspace_bytes(mode, chunk), dtype=torch.uint8, device=cuda)
    dp.reset()
    dp.run(mode, 0, prog.num_slices, workspace=ws)
    got = float(dp.result())
    want = float(load_golden("vc60_s4")["reference"]["bigint"])
    assert rel(got, want) <= (PLAIN_TOL if mode == runtime.MODE_F64 else SPLIT_TOL)
    # a second run accumulates onto the first
    dp.run(mode, 0, prog.num_slices, workspace=ws)
    assert rel(float(dp.result()), 2 * want) <= (PLAIN_TOL if mode == runtime.MODE_F64 else SPLIT_TOL)
    dp.close()


def test_workspace_too_small_is_out_of_memory(cuda):
    import torch

    prog = program("wvc120")
    dp = runtime.DeviceProgram(prog)
    ws = torch.empty(64, dtype=torch.uint8, device=cuda)
    with pytest.raises(runtime.DeviceOutOfMemory):
        dp.run(runtime.MODE_F64, 0, 1, workspace=ws)
    dp.close()


@pytest.mark.parametrize("name", ["wvc30_s3", "r3cnf20_factor", "vc50_bundled"])
def test_plugin_contract_sliced_on_plan_objects(name, cuda):
    doc = load_golden(name)
    plan = FakePlan(program(name))
    got = float(api.GB300API().contract_sliced(plan))
    assert rel(got, doc["reference"]["float64"]) <= PLAIN_TOL
    got = float(api.GB300API().contract_sliced(plan, num_slice_limit=1))
    if "prefix_float64" in doc["reference"]:
        assert abs(got - doc["reference"]["prefix_float64"][0]) <= PLAIN_TOL * abs(doc["reference"]["float64"])


def test_plugin_contract_single_network(cuda):
    doc = load_golden("vc50_seed0")
    plan = FakePlan(program("vc50_seed0"))
    res = api.GB300API().contract(plan.network, plan.tree)
    assert rel(float(res[()]), doc["reference"]["float64"]) <= PLAIN_TOL


def test_per_join_timing(cuda):
    prog = program("wvc120")
    dp = runtime.DeviceProgram(prog)
    dp.set_timing(True)
    dp.reset()
    dp.run(runtime.MODE_F64)
    t = dp.join_times()
    assert t.shape == (prog.num_joins,) and np.all(t >= 0) and t.sum() > 0
    assert rel(float(dp.result()), load_golden("wvc120")["reference"]["float64"]) <= PLAIN_TOL
    dp.close()


def _workload(name):
    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", name + ".json.gz"), "rt") as f:
        return json.load(f)


@pytest.mark.parametrize("mode,tol", [(runtime.MODE_F64, PLAIN_TOL), (runtime.MODE_SPLIT, SPLIT_TOL)])
def test_weighted_cubic_vc_220_sliced_1024(mode, tol, cuda):
    doc = _workload("wvc220_s10")
    prog = Program.from_dict(doc["program"])
    got = float(api.GB300API(mode=mode).contract_program(prog))
    assert rel(got, doc["reference"]["float64"]) <= tol


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("mode", [runtime.MODE_F64, runtime.MODE_SPLIT])
def test_leaves_built_on_device_match_uploaded_leaves(name, mode, cuda):
    """Clause and variable leaves built by the library from their parameters
    (togb_program_create_compact) give exactly the count of the same program
    with every leaf's dense values uploaded (togb_program_create)."""
    prog = program(name)
    got = []
    for leaves in ("device", "host"):
        dp = runtime.DeviceProgram(prog, leaves=leaves)
        dp.reset()
        dp.run(mode)
        got.append(dp.result().copy())
        dp.close()
    assert np.array_equal(got[0], got[1])
