"""The int form's checker, pinned on the CPU (no GPU).

* The oracle in int64 gives the reference's own ``bigint`` counts of the
  unweighted fixtures (made by running the reference with
  ``--entry_type bigint``; they fit 64 bits).
* Where counts exceed 2^64 (integer weights 3 and 5), the oracle's int64
  count is the exact integer count modulo 2^64, as numpy int64 / uint64
  tensors give it (``numpy_apis.py:15-22``).
* Leaf values are converted toward zero, numpy's float-to-int64 cast.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from intcases import MOD, exact_count, integer_weights, oracle_words
from tensororder_gb300.program import Program

BIGINT = [n for n in golden_names() if "bigint" in load_golden(n)["reference"]]


def test_unweighted_fixtures_carry_bigint_counts():
    assert set(BIGINT) >= {"vc50_bundled", "vc50_seed0", "vc60_s4"}


@pytest.mark.parametrize("name", BIGINT)
def test_oracle_int64_equals_reference_bigint(name):
    doc = load_golden(name)
    prog = Program.from_dict(doc["program"])
    assert int(oracle_words(prog)) == int(doc["reference"]["bigint"])


@pytest.mark.parametrize("name", golden_names())
def test_oracle_int64_wraps_modulo_2_64(name):
    prog = integer_weights(Program.from_dict(load_golden(name)["program"]))
    assert int(oracle_words(prog)) == exact_count(prog) % MOD


def test_wrapping_cases_exceed_64_bits():
    big = [n for n in golden_names()
           if exact_count(integer_weights(Program.from_dict(load_golden(n)["program"]))) >= MOD]
    assert len(big) >= 5


def test_leaf_values_convert_toward_zero():
    v = np.array([0.7, -0.7, 2.5, -2.5, 3.0, 1e15 + 0.5])
    assert v.astype(np.int64).tolist() == [0, 0, 2, -2, 3, 10 ** 15]
    assert np.array_equal(v.astype(np.int64), np.trunc(v).astype(np.int64))
