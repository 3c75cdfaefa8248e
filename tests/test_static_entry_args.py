"""Argument checks of ``runtime.contract_static_f64`` (no GPU needed).

The allocation-free entry point receives raw device addresses and sizes every
buffer from the program alone, so the host wrapper must reject a buffer of the
wrong type, layout, size or device before anything is queued.  These cases
run on CPU tensors: every check fires before the library is called.
"""
import numpy as np
import pytest
import torch

from conftest import load_golden
from tensororder_gb300 import runtime
from tensororder_gb300.program import Program


@pytest.fixture(scope="module")
def prog():
    return Program.from_dict(load_golden("wvc30_s3")["program"])


def n_values(prog):
    return sum(1 << l.rank for l in prog.leaves)


def test_root_rank_of_a_count_is_zero(prog):
    assert runtime.program_root_rank(prog) == 0


@pytest.mark.parametrize("case", ["leaf_dtype", "out_dtype", "leaf_strided", "out_size", "leaf_short", "cpu"])
def test_mismatch_raises_before_launch(prog, case, monkeypatch):
    called = []
    monkeypatch.setattr(runtime, "_contract_static_f64", lambda *a: called.append(a))
    leaves = torch.zeros(n_values(prog), dtype=torch.float64)
    out = torch.zeros(1, dtype=torch.float64)
    if case == "leaf_dtype":
        leaves = leaves.float()
    elif case == "out_dtype":
        out = out.float()
    elif case == "leaf_strided":
        leaves = torch.zeros(2 * n_values(prog), dtype=torch.float64)[::2]
    elif case == "out_size":
        out = torch.zeros(2, dtype=torch.float64)
    elif case == "leaf_short":
        leaves = leaves[:-1]
    with pytest.raises(ValueError):
        runtime.contract_static_f64(prog, leaves, out)
    assert not called


def test_non_tensor_rejected(prog):
    with pytest.raises(ValueError):
        runtime.contract_static_f64(prog, np.zeros(n_values(prog)), torch.zeros(1, dtype=torch.float64))
