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
