"""Uneven batches in one CUDA graph (togb_batch): every instance of a mixed
batch -- the golden plans, sliced and unsliced, line- and factor-Flow -- gets
its reference count (plain 1e-12, split 1e-6), on repeated steps, with and
without autotuned kernels."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from tensororder_gb300 import batch, runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu

NAMES = golden_names()


def programs_and_counts(repeat=1):
    progs, want = [], []
    for _ in range(repeat):
        for n in NAMES:
            doc = load_golden(n)
            progs.append(Program.from_dict(doc["program"]))
            want.append(float(doc["reference"]["float64"]))
    return progs, np.array(want)


@pytest.mark.parametrize("mode,tol", [(runtime.MODE_F64, 1e-12), (runtime.MODE_SPLIT, 1e-6)])
@pytest.mark.parametrize("nstreams", [1, 4])
def test_batch_counts_match_reference(mode, tol, nstreams, cuda):
    progs, want = programs_and_counts(repeat=2)
    ex = batch.BatchExecutor(progs, mode, nstreams=nstreams)
    for _ in range(3):
        ex.run()
        got = ex.counts()
        assert np.all(np.abs(got - want) <= tol * np.abs(want))
    ex.close()


@pytest.mark.parametrize("mode,tol", [(runtime.MODE_F64, 1e-12), (runtime.MODE_SPLIT, 1e-6)])
def test_autotuned_batch_keeps_counts(mode, tol, cuda):
    progs, want = programs_and_counts()
    tuner = batch.Autotuner(mode)
    assert tuner.tune(progs[:4]) > 0
    ex = batch.BatchExecutor(progs, mode, nstreams=4, tuner=tuner)
    ex.run()
    got = ex.counts()
    ex.close()
    assert np.all(np.abs(got - want) <= tol * np.abs(want))


def test_batch_rejects_duplicate_program(cuda):
    import ctypes

    prog = Program.from_dict(load_golden("wvc18_s2")["program"])
    dp = runtime.DeviceProgram(prog)
    ws = dp.allocate_workspace(runtime.MODE_F64, dp.num_slices)
    h = (ctypes.c_void_p * 2)(dp._h.value, dp._h.value)
    p = (ctypes.c_void_p * 2)(ws.data_ptr(), ws.data_ptr())
    b = (ctypes.c_size_t * 2)(ws.numel(), ws.numel())
    out = ctypes.c_void_p()
    st = runtime.lib().togb_batch_create(h, 2, runtime.MODE_F64, p, b, 1, ctypes.byref(out))
    assert st == runtime.ERR_INVALID and not out.value
    dp.close()


def test_batch512_every_instance_matches_reference(cuda):
    """The 512-instance uneven batch (config 4) in the split form: the 291
    instances with the reference's full count are checked on the batch's
    counts, the other 221 on the reference's count of their first slices
    (contracted separately), all within 1e-6.  The plain form is checked on
    the prefixes of the cheaper instances within 1e-12."""
    import os

    from conftest import ROOT
    from tensororder_gb300.run_batch import load, reference_errors

    progs, refs, items = load(os.path.join(ROOT, "tensororder_gb300", "plans", "batch512.json.gz"))
    ex = batch.BatchExecutor(progs, runtime.MODE_SPLIT, nstreams=16)
    ex.run()
    counts = ex.counts()
    ex.close()
    full, prefix = reference_errors(progs, items, counts, runtime.MODE_SPLIT)
    assert full.size + prefix.size == 512
    assert full.max() <= 1e-6 and prefix.max() <= 1e-6
    _, prefix64 = reference_errors(progs, items, np.full(len(progs), np.nan), runtime.MODE_F64,
                                   max_prefix_flops=2e10)
    assert prefix64.size >= 100 and prefix64.max() <= 1e-12
