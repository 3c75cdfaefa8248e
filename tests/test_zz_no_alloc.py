"""togb_contract_static_f64: the entry point that allocates no device memory.

It exists for callers that cannot call cudaMalloc -- a process whose device
memory is all owned by its own allocator, or a pipeline that cannot take the
device-wide synchronisation of cudaMalloc/cudaFree.  These tests call it
through the C ABI with caller-owned input and output buffers and check it
against the allocating entry point (togb_program_*) and against the
reference's own numpy FP64 count recorded in the golden fixture, within the
plain-form tolerance, twice in a row, since every call reuses the same static
scratch.  This file sorts last so a failure here leaves the rest of the suite
already run.
"""
import numpy as np
import pytest

from conftest import load_golden
from tensororder_gb300 import runtime
from tensororder_gb300.program import Leaf, Program

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.mark.parametrize("name", ["vc60_s4", "wvc30_s3", "wvc120", "r3cnf20_factor"])
def test_static_entry_matches_allocating_entry(name, cuda):
    import torch

    doc = load_golden(name)
    prog = Program.from_dict(doc["program"])
    reference = doc["reference"]["float64"]
    dp = runtime.DeviceProgram(prog)
    dp.reset()
    dp.run(runtime.MODE_F64)
    want = dp.result().reshape(-1)
    leaves = torch.as_tensor(dp._values, device=cuda)  # owned by the caller
    out = torch.empty(1 << int(dp.info.root_rank), dtype=torch.float64, device=cuda)
    dp.close()
    for _ in range(2):
        out.fill_(float("nan"))
        runtime.contract_static_f64(prog, leaves, out)
        got = out.cpu().numpy()
        assert np.all(np.abs(got - want) <= TOL * np.abs(want))
        assert abs(got[0] - reference) <= TOL * abs(reference)


def test_static_entry_rejects_programs_beyond_its_scratch(cuda):
    import torch

    # Two rank-12 tensors with no shared edge: their outer product has rank
    # 24, i.e. 128 MiB per slice, beyond the 32 MiB static scratch; two more
    # leaves contract it back to a count.
    ones = np.ones((2,) * 12)
    a = Leaf(list(range(12)), "dense", values=ones)
    b = Leaf(list(range(12, 24)), "dense", values=ones)
    c = Leaf(list(range(12)), "dense", values=ones)
    d = Leaf(list(range(12, 24)), "dense", values=ones)
    prog = Program([a, b, c, d], [0, 1, -1, 2, -1, 3, -1])
    leaves = torch.ones(4 << 12, dtype=torch.float64, device=cuda)
    out = torch.empty(1, dtype=torch.float64, device=cuda)
    with pytest.raises(runtime.DeviceOutOfMemory) as exc:
        runtime.contract_static_f64(prog, leaves, out)
    assert "static scratch" in str(exc.value)
    assert str(runtime.STATIC_SCRATCH_BYTES) in str(exc.value)
