"""Exact counts for the ``bigint`` entry type, on the host (no GPU).

``tensororder_gb300.exact`` recovers an integer from its residue modulo 2^64
(the int form) and modulo primes below 2^28 (the residue form), sized by a
floating-point bound.  The plugin's orchestration is checked with a stand-in
device program whose forms report residues of a known integer.
"""
import random

import numpy as np
import pytest

from conftest import golden_names, load_golden
from intcases import integer_weights
from tensororder_gb300 import api, exact, runtime
from tensororder_gb300.program import Leaf, Program


def test_moduli_are_distinct_primes_below_2_28():
    sympy = pytest.importorskip("sympy")
    assert len(set(exact.MODULI)) == len(exact.MODULI) == 64
    assert all(p < (1 << 28) and sympy.isprime(p) for p in exact.MODULI)
    rng = random.Random(7)
    for _ in range(20000):
        n = rng.randrange(1, 1 << 31)
        assert exact._is_prime(n) == sympy.isprime(n)


@pytest.mark.parametrize("bits", [1, 40, 63, 64, 65, 120, 300, 1000, 1020])
def test_combine_recovers_signed_integers(bits):
    rng = random.Random(bits)
    for _ in range(50):
        x = rng.randrange(1 << bits) * rng.choice([1, -1])
        moduli = exact.moduli_for(float(abs(x)) * (1 + 1e-9) + 1)
        got = exact.combine(x % exact.WORD, [x % p for p in moduli], moduli)
        assert got == x


def test_moduli_for_takes_the_fewest_primes():
    for bound in [0.0, 1.0, 2.0 ** 62, 2.0 ** 63, 2.0 ** 100, 2.0 ** 700]:
        ms = exact.moduli_for(bound)
        M = exact.WORD
        for p in ms:
            M *= p
        assert M > 2 * int(bound) + 1
        if ms:
            assert M // ms[-1] <= 2 * int(bound) + 2
    with pytest.raises(OverflowError):
        exact.moduli_for(float("inf"))


def test_leaf_classification():
    for name in golden_names():
        prog = Program.from_dict(load_golden(name)["program"])
        unweighted = load_golden(name)["weights"] == "unweighted"
        assert exact.integer_leaves(prog) == (unweighted or all(l.kind != "var" for l in prog.leaves))
        assert exact.integer_leaves(integer_weights(prog))


def test_negative_weights_are_refused_before_any_device_work():
    neg = integer_weights(Program.from_dict(load_golden("vc50_bundled")["program"]), -2, 3)
    with pytest.raises(runtime.TogbError, match="non-negative"):
        runtime.DeviceProgram(neg)


class Info:
    flops_per_slice = 1e6
    root_rank = 0


class ResidueProgram:
    """Stands in for a DeviceProgram whose count is the integer X: the
    floating forms report float(X), the int form X mod 2^64, the residue form
    X mod p."""

    X = 0
    made = []

    def __init__(self, program, device=0):
        self.info = Info()
        self.program = program
        self.modulus = None
        self.mode = None
        self.calls = []
        self.ranges = []
        ResidueProgram.made.append(self)

    def set_leaves(self, program, stream=None):
        self.program = program

    def close(self):
        pass

    def reset(self, stream=None):
        self.mode = None

    def allocate_workspace(self, mode, slices, max_fraction=0.5):
        return None

    def run(self, mode, begin=0, end=None, workspace=None, stream=None):
        self.mode = mode
        self.calls.append((mode, self.modulus))
        self.ranges.append((mode, begin, end))

    def set_modulus(self, p):
        self.modulus = p

    def _value(self):
        return self.X

    def result(self, stream=None):
        assert self.mode in (runtime.MODE_F64, runtime.MODE_SPLIT)
        return np.array(float(self._value()))

    def result_words(self, stream=None, dtype=np.int64):
        if self.mode == runtime.MODE_INT64:
            w = self._value() % exact.WORD
        else:
            assert self.mode == runtime.MODE_MOD
            w = self._value() % self.modulus
        return np.array(w, dtype=np.uint64).view(dtype)


@pytest.fixture
def fake(monkeypatch):
    ResidueProgram.made = []
    monkeypatch.setattr(runtime, "DeviceProgram", ResidueProgram)
    monkeypatch.setattr(api.GB300API, "_stream", lambda self: None)
    monkeypatch.setattr(api.GB300API, "_wait", staticmethod(lambda stream: None))
    return ResidueProgram


def small_network(w_neg=3.0, w_pos=5.0, groups=0):
    leaves = [Leaf([0, 1], "or", positive=[True, False]), Leaf([0], "var", w_neg=w_neg, w_pos=w_pos),
              Leaf([1], "var", w_neg=2.0, w_pos=7.0)]
    tokens = [0, 1, -1, 2, -1]
    for i in range(groups):  # independent variables, one slice group each
        leaves.append(Leaf([2 + i], "var", w_neg=1.0, w_pos=1.0))
        tokens += [3 + i, -1]
    return Program(leaves, tokens, [[2 + i] for i in range(groups)]).validate()


@pytest.mark.parametrize("x", [0, 12345, (1 << 64) + 17, 3 ** 200, 7 ** 350 + 1])
def test_plugin_reconstructs_the_count(fake, x):
    fake.X = x
    backend = api.GB300API()
    backend.add_argument("entry_type", "bigint")
    got = backend.contract_program(small_network())
    assert type(got) is int and got == x
    calls = fake.made[0].calls
    assert calls[0] == (runtime.MODE_SPLIT, None) and calls[1][0] == runtime.MODE_INT64
    moduli = [m for mode, m in calls[2:]]
    assert moduli == exact.moduli_for(float(x) * (1 + 1e-4) + 1)


def test_plugin_non_integer_leaves_give_the_fp64_count(fake):
    fake.X = 7
    backend = api.GB300API()
    backend.add_argument("entry_type", "bigint")
    got = backend.contract_program(small_network(w_neg=0.25))
    assert type(got) is float and got == 7.0
    assert [m for m, _ in fake.made[0].calls] == [runtime.MODE_F64]


def test_every_pass_honours_the_slice_limit(fake):
    """``num_slice_limit`` keeps a prefix of the slices (``base_api.py:23-24``):
    the bound, the int form and every residue pass cover the same prefix."""
    fake.X = 3 ** 100
    prog = small_network(groups=3)  # 8 slices
    backend = api.GB300API()
    backend.add_argument("entry_type", "bigint")
    backend.slices_per_call = 2
    backend.contract_program(prog, num_slice_limit=5)
    ranges = fake.made[0].ranges
    modes = sorted(set(m for m, _, _ in ranges))
    assert runtime.MODE_SPLIT in modes and runtime.MODE_INT64 in modes and runtime.MODE_MOD in modes
    for mode in (runtime.MODE_SPLIT, runtime.MODE_INT64):
        mine = [(b, e) for m, b, e in ranges if m == mode]
        assert mine[0][0] == 0 and mine[-1][1] == 5
        assert all(e1 == b2 for (_, e1), (b2, _) in zip(mine, mine[1:]))
