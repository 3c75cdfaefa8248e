"""Counting the same network again with other weights (togb_program_set_leaves).

A device program keeps its lowering, layouts and workspace; new clause and
variable parameters and dense values are uploaded and the leaves rebuilt on
the device.  The count must equal a freshly created program's bit for bit and
the oracle's within the form's tolerance, also when a leaf's power-of-two
normaliser changes (weights scaled by 8) and back again.  The plugin keeps its
last program and reuses it for a count of the same structure."""
import copy

import numpy as np
import pytest

from conftest import load_golden
from oracle import contract as oracle
from tensororder_gb300 import api, runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu

MODES = [(runtime.MODE_F64, 1e-12), (runtime.MODE_SPLIT, 1e-6)]


def reweighted(prog, seed, scale=1.0):
    """The same network with new variable weights (scaled) and, for dense
    leaves, new values; clause polarities unchanged."""
    rng = np.random.default_rng(seed)
    out = copy.deepcopy(prog)
    for l in out.leaves:
        if l.kind == "var":
            l.w_neg = float(rng.uniform(0.2, 0.8)) * scale
            l.w_pos = float(rng.uniform(0.2, 0.8)) * scale
        elif l.kind == "dense":
            l.values = rng.uniform(0.5, 1.5, size=np.shape(l.values)) * scale
    return out


def count(dp, mode):
    dp.reset()
    dp.run(mode)
    return float(dp.result().reshape(-1)[0])


def want(prog):
    return float(sum(oracle.contract(prog, s)[0] for s in range(prog.num_slices)))


@pytest.mark.parametrize("name", ["wvc30_s3", "r3cnf20_factor", "wvc120"])
@pytest.mark.parametrize("mode,tol", MODES)
def test_new_weights_give_a_fresh_programs_count(name, mode, tol, cuda):
    p1 = Program.from_dict(load_golden(name)["program"])
    variants = [reweighted(p1, 1), reweighted(p1, 2, scale=8.0), p1]
    dp = runtime.DeviceProgram(p1)
    first = count(dp, mode)
    count(dp, mode)  # a second run: the phases are captured as graphs
    for q in variants:
        dp.set_leaves(q)
        got = count(dp, mode)
        fresh = runtime.DeviceProgram(q)
        ref = count(fresh, mode)
        fresh.close()
        assert got == ref
        w = want(q)
        assert abs(got - w) <= tol * abs(w)
    assert got == first  # back to the original weights
    dp.close()


def test_a_changed_leaf_kind_is_rejected(cuda):
    p1 = Program.from_dict(load_golden("wvc30_s3")["program"])
    p2 = copy.deepcopy(p1)
    i = next(i for i, l in enumerate(p2.leaves) if l.kind == "var")
    l = p2.leaves[i]
    l.kind, l.values = "dense", l.parent()
    dp = runtime.DeviceProgram(p1)
    with pytest.raises(runtime.TogbError) as e:
        dp.set_leaves(p2)
    assert e.value.status == runtime.ERR_INVALID
    # the program is untouched and still counts p1
    w = want(p1)
    assert abs(count(dp, runtime.MODE_F64) - w) <= 1e-12 * abs(w)
    dp.close()


def test_plugin_reuses_its_program_for_the_same_structure(cuda):
    p1 = Program.from_dict(load_golden("wvc120")["program"])
    p2 = reweighted(p1, 3)
    backend = api.GB300SplitAPI()
    c1 = float(backend.contract_program(p1))
    dp = backend.last_program
    c2 = float(backend.contract_program(p2))
    assert backend.last_program is dp
    for c, q in ((c1, p1), (c2, p2)):
        w = want(q)
        assert abs(c - w) <= 1e-6 * abs(w)
    other = Program.from_dict(load_golden("wvc30_s3")["program"])
    backend.contract_program(other)
    assert backend.last_program is not dp
