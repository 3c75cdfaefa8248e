"""Exact counts on the device: the residue form (TOGB_MODE_MOD) and the
``bigint`` entry type built on it.

The reference's ``bigint`` entry type contracts Python integers
(``numpy_apis.py:15-22``).  Here the count comes from the int form (modulo
2^64) and residue-form counts modulo primes below 2^28, combined by the
Chinese remainder theorem.  Every check is exact:

* every golden plan with integer weights against the Python-integer oracle
  (counts of 44 to 335 bits), and the unweighted fixtures against the
  reference's own ``bigint`` counts;
* fractional weights give the plain FP64 count, as Python floats;
* every kernel a join may run gives the same residue;
* n=220 (unweighted, 1024 slices): the exact count agrees with the int
  form's word, the plain FP64 count, and a residue modulo a prime it was
  not built from;
* the modulus rules of the accumulator.
"""
import gzip
import json
import os

import numpy as np
import pytest

from conftest import golden_names, load_golden
from intcases import MOD, exact_count, integer_weights
from tensororder_gb300 import api, exact, runtime
from tensororder_gb300.program import Program

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIGINT = [n for n in golden_names() if "bigint" in load_golden(n)["reference"]]


def program(name):
    return Program.from_dict(load_golden(name)["program"])


def bigint_backend():
    backend = api.GB300API()
    backend.add_argument("entry_type", "bigint")
    return backend


def residue(dp, p, begin=0, end=None):
    dp.set_modulus(p)
    dp.reset()
    dp.run(runtime.MODE_MOD, begin, end)
    return int(dp.result_words(dtype=np.uint64).reshape(-1)[0])


@pytest.mark.parametrize("name", golden_names())
def test_bigint_count_is_exact(name, cuda):
    prog = integer_weights(program(name))
    got = bigint_backend().contract_program(prog)
    assert type(got) is int
    assert got == exact_count(prog)


@pytest.mark.parametrize("name", BIGINT)
def test_bigint_equals_the_references_bigint(name, cuda):
    doc = load_golden(name)
    got = bigint_backend().contract_program(Program.from_dict(doc["program"]))
    assert type(got) is int and got == int(doc["reference"]["bigint"])


def test_bigint_fractional_weights_give_the_fp64_count(cuda):
    prog = program("wvc30_s3")
    got = bigint_backend().contract_program(prog)
    plain = float(api.GB300API().contract_program(prog))
    assert type(got) is float and got == plain


@pytest.mark.parametrize("name", ["wvc120", "vc60_s4", "r3cnf20_factor", "wvc30_s3", "r3cnf16_line"])
@pytest.mark.parametrize("kernel", [0, 1, 2])
def test_every_kernel_gives_the_same_residue(name, kernel, cuda):
    prog = integer_weights(program(name))
    p = exact.MODULI[5]
    dp = runtime.DeviceProgram(prog)
    for j, ks in enumerate(dp.allowed_kernels(runtime.MODE_MOD)):
        assert 3 not in ks
        if kernel in ks:
            dp.set_kernel(runtime.MODE_MOD, j, kernel)
    got = residue(dp, p)
    dp.close()
    assert got == exact_count(prog) % p


def test_n220_exact_count_is_consistent(cuda):
    with gzip.open(os.path.join(ROOT, "tensororder_gb300", "plans", "wvc220_s10.json.gz"), "rt") as f:
        doc = json.load(f)
    prog = integer_weights(Program.from_dict(doc["program"]), 1, 1)  # unweighted
    backend = bigint_backend()
    x = backend.contract_program(prog)
    dp = backend.last_program
    dp.reset()
    dp.run(runtime.MODE_INT64)
    word = int(dp.result_words(dtype=np.uint64).reshape(-1)[0])
    q = exact.MODULI[-1]  # far past the primes a 2^140 count uses
    rq = residue(dp, q)
    plain = float(api.GB300API().contract_program(prog))
    assert x.bit_length() > 100
    assert x % MOD == word
    assert x % q == rq
    assert abs(float(x) - plain) <= 1e-12 * float(x)


def test_modulus_rules(cuda):
    prog = integer_weights(program("wvc30_s3"))
    want = exact_count(prog)
    p1, p2 = exact.MODULI[0], exact.MODULI[1]
    dp = runtime.DeviceProgram(prog)
    with pytest.raises(runtime.TogbError):
        dp.run(runtime.MODE_MOD)  # no modulus yet
    for bad in (0, 1, 1 << 28):
        with pytest.raises(runtime.TogbError):
            dp.set_modulus(bad)
    S = prog.num_slices
    dp.set_modulus(p1)
    dp.reset()
    dp.run(runtime.MODE_MOD, 0, S // 2)
    dp.set_modulus(p2)
    with pytest.raises(runtime.TogbError):
        dp.run(runtime.MODE_MOD, S // 2, S)  # the accumulator holds residues modulo p1
    with pytest.raises(runtime.TogbError):
        dp.run(runtime.MODE_INT64)
    dp.set_modulus(p1)
    dp.run(runtime.MODE_MOD, S // 2, S)
    r1 = int(dp.result_words(dtype=np.uint64).reshape(-1)[0])
    r2 = residue(dp, p2)
    dp.close()
    assert r1 == want % p1 and r2 == want % p2
