"""The int form on the device (TOGB_MODE_INT64, ``--entry_type int`` / ``uint``).

The reference contracts numpy int64 / uint64 tensors for these entry types
(``numpy_apis.py:15-22``): sums and products modulo 2^64.  Integer sums are
exact in any order, so every check here is bit for bit:

* unweighted fixtures: the reference's own ``bigint`` counts;
* integer weights 3 and 5 (counts far beyond 2^64): the oracle in int64, with
  leaves built on the device or uploaded;
* every kernel a join may run (thread-per-output, tiled, reduction) gives the
  same words;
* n=220 sliced 1024 ways (unweighted): slice ranges and chunkings add up to
  the full count modulo 2^64, and its first slice equals the oracle's;
* new weights through ``set_leaves``, and the accumulator's kind checks.
"""
import gzip
import json
import os

import numpy as np
import pytest

from conftest import golden_names, load_golden
from intcases import MOD, integer_weights, oracle_words
from oracle import contract as oracle
from tensororder_gb300 import api, runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu

MODE = runtime.MODE_INT64
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIGINT = [n for n in golden_names() if "bigint" in load_golden(n)["reference"]]


def program(name):
    return Program.from_dict(load_golden(name)["program"])


def words(dp, begin=0, end=None, workspace=None):
    dp.reset()
    dp.run(MODE, begin, end, workspace=workspace)
    return dp.result_words(dtype=np.uint64).reshape(-1)[0]


@pytest.mark.parametrize("name", BIGINT)
@pytest.mark.parametrize("entry,word", [("int", np.int64), ("uint", np.uint64)])
def test_plugin_count_equals_reference_bigint(name, entry, word, cuda):
    doc = load_golden(name)
    backend = api.GB300API()
    backend.add_argument("entry_type", entry)
    got = backend.contract_program(Program.from_dict(doc["program"]))
    assert isinstance(got, word)
    assert int(got) == int(doc["reference"]["bigint"])


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("leaves", ["device", "host"])
def test_counts_wrap_like_numpy_int64(name, leaves, cuda):
    prog = integer_weights(program(name))
    dp = runtime.DeviceProgram(prog, leaves=leaves)
    got = words(dp)
    dp.close()
    assert got == oracle_words(prog)


@pytest.mark.parametrize("name", ["wvc120", "vc60_s4", "r3cnf20_factor", "wvc30_s3", "r3cnf16_line"])
@pytest.mark.parametrize("kernel", [0, 1, 2])
def test_every_kernel_gives_the_same_words(name, kernel, cuda):
    prog = integer_weights(program(name))
    dp = runtime.DeviceProgram(prog)
    allowed = dp.allowed_kernels(MODE)
    assert all(3 not in ks for ks in allowed)  # no tensor-core kernel in the int form
    changed = 0
    for j, ks in enumerate(allowed):
        if kernel in ks:
            dp.set_kernel(MODE, j, kernel)
            changed += 1
    got = words(dp)
    info = dp.joins(MODE)
    dp.close()
    assert got == oracle_words(prog)
    assert sum(1 for j in range(len(allowed)) if int(info[j][3]) == kernel) >= changed


def _wvc220_unweighted():
    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", "wvc220_s10.json.gz"), "rt") as f:
        doc = json.load(f)
    return integer_weights(Program.from_dict(doc["program"]), 1, 1)


def test_n220_slice_ranges_and_chunks_add_up(cuda):
    import torch

    prog = _wvc220_unweighted()
    S = prog.num_slices
    dp = runtime.DeviceProgram(prog)
    full = words(dp)
    halves = (int(words(dp, 0, S // 2)) + int(words(dp, S // 2, S))) % MOD
    # two calls into one accumulator, and a workspace of 96 slices per chunk
    dp.reset()
    dp.run(MODE, 0, 300)
    dp.run(MODE, 300, S)
    two_calls = dp.result_words(dtype=np.uint64).reshape(-1)[0]
    ws = torch.empty(dp.workspace_bytes(MODE, 96), dtype=torch.uint8, device=cuda)
    chunked = words(dp, workspace=ws)
    first = words(dp, 0, 1)
    dp.close()
    assert int(full) == halves == int(two_calls) == int(chunked)
    assert full != 0
    assert first == oracle_words(prog, 1)


def test_new_weights_reconvert_the_int_leaves(cuda):
    base = program("wvc30_s3")
    p1, p2 = integer_weights(base, 3, 5), integer_weights(base, 2, 7)
    dp = runtime.DeviceProgram(p1)
    a = words(dp)
    dp.set_leaves(p2)
    b = words(dp)
    dp.set_leaves(p1)
    c = words(dp)
    dp.close()
    assert a == oracle_words(p1) and b == oracle_words(p2) and c == a
    assert a != b


def test_one_kind_of_sum_between_resets(cuda):
    prog = integer_weights(program("vc60_s4"))
    dp = runtime.DeviceProgram(prog)
    dp.reset()
    dp.run(runtime.MODE_F64)
    f = float(dp.result().reshape(-1)[0])
    with pytest.raises(runtime.TogbError):
        dp.run(MODE)  # the accumulator holds FP64 sums
    with pytest.raises(runtime.TogbError):
        dp.result_words()
    w = words(dp)
    with pytest.raises(runtime.TogbError):
        dp.result()
    with pytest.raises(runtime.TogbError):
        dp.run(runtime.MODE_SPLIT)
    dp.run(MODE)  # a second count into the same words
    twice = dp.result_words(dtype=np.uint64).reshape(-1)[0]
    dp.close()
    assert w == oracle_words(prog)
    assert int(twice) == (2 * int(w)) % MOD
    assert abs(f - float(oracle.contract_sliced(prog))) <= 1e-12 * abs(f)


def _word_case(rng, ra, rb, k):
    """Random int64 tensors spanning the whole range, so products and sums wrap."""
    a = rng.integers(-(1 << 63), (1 << 63) - 1, size=(2,) * ra, dtype=np.int64, endpoint=True)
    b = rng.integers(-(1 << 63), (1 << 63) - 1, size=(2,) * rb, dtype=np.int64, endpoint=True)
    return a, b, (list(rng.permutation(ra)[:k]), list(rng.permutation(rb)[:k]))


def _check_words(a, b, axes, cuda):
    import torch

    want = np.tensordot(a, b, axes)
    got = runtime.tensordot_i64(torch.as_tensor(a, device=cuda), torch.as_tensor(b, device=cuda), axes)
    got = got.cpu().numpy()
    assert got.dtype == np.int64 and got.shape == want.shape
    assert np.array_equal(got, want)


@pytest.mark.parametrize("seed", range(24))
def test_tensordot_i64_wraps_like_numpy(seed, cuda):
    rng = np.random.default_rng(1000 + seed)
    ra, rb = int(rng.integers(0, 10)), int(rng.integers(0, 10))
    k = int(rng.integers(0, min(ra, rb) + 1))
    _check_words(*_word_case(rng, ra, rb, k), cuda)


@pytest.mark.parametrize("ra,rb,k", [(10, 10, 5), (16, 16, 8), (14, 12, 6), (20, 14, 10), (12, 20, 4),
                                     (8, 8, 0), (12, 12, 12)])
def test_tensordot_i64_shapes(ra, rb, k, cuda):
    rng = np.random.default_rng(ra * 1000 + rb * 10 + k)
    _check_words(*_word_case(rng, ra, rb, k), cuda)


@pytest.mark.parametrize("entry,dtype", [("int", np.int64), ("uint", np.uint64)])
def test_plugin_tensordot_follows_the_entry_type(entry, dtype, cuda):
    rng = np.random.default_rng(5)
    a = rng.integers(0, np.iinfo(dtype).max, size=(2,) * 7, dtype=dtype, endpoint=True)
    b = rng.integers(0, np.iinfo(dtype).max, size=(2,) * 6, dtype=dtype, endpoint=True)
    axes = ([1, 4, 6], [5, 0, 2])
    backend = api.GB300API()
    backend.add_argument("entry_type", entry)
    got = backend.tensordot(a, b, axes).cpu().numpy().view(dtype)
    assert np.array_equal(got, np.tensordot(a, b, axes))
