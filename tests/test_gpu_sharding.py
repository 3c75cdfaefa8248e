"""Slice sharding on the GPU: the slice blocks of 1..4 ranks, contracted one
after another on this GPU through ``sharding.device_range_runner`` and
combined, give the reference's count (plain form <= 1e-12, split <= 1e-6)."""
import numpy as np
import pytest

from conftest import load_golden
from tensororder_gb300 import runtime, sharding
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [1, 2, 3, 4])
@pytest.mark.parametrize("mode,tol", [(runtime.MODE_F64, 1e-12), (runtime.MODE_SPLIT, 1e-6)])
def test_device_shards_combine_to_the_count(world, mode, tol, cuda):
    doc = load_golden("vc60_s4")
    prog = Program.from_dict(doc["program"])
    dp = runtime.DeviceProgram(prog)
    run = sharding.device_range_runner(dp, mode)
    parts = [run(*sharding.slice_range(prog.num_slices, r, world)) for r in range(world)]
    got = float(sharding.combine(parts)[0])
    dp.close()
    want = float(doc["reference"]["float64"])
    assert abs(got - want) <= tol * want


@pytest.mark.parametrize("world", [1, 3, 5])
@pytest.mark.parametrize("mode", [runtime.MODE_INT64, runtime.MODE_MOD])
def test_device_word_shards_combine_exactly(world, mode, cuda):
    """The int forms shard exactly: the words of 1, 3 and 5 slice blocks,
    combined modulo 2^64 (int form) or the prime (residue form), equal the
    whole count's, and with a Python-integer oracle."""
    from intcases import MOD, exact_count, integer_weights

    prog = integer_weights(Program.from_dict(load_golden("vc60_s4")["program"]))
    p = 268435399
    dp = runtime.DeviceProgram(prog)
    dp.set_modulus(p)
    run = sharding.device_words_runner(dp, mode)
    parts = [run(*sharding.slice_range(prog.num_slices, r, world)) for r in range(world)]
    modulus = p if mode == runtime.MODE_MOD else 0
    got = int(np.ravel(sharding.combine_words(parts, modulus))[0])
    dp.close()
    assert got == exact_count(prog) % (modulus or MOD)
