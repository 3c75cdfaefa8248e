"""The numpy oracle against the golden vectors made by the reference itself
(tests/golden/make_golden.py): FP64 counts, exact bigint counts, brute-force
counts and slice-prefix counts (num_slice_limit)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import contract as oracle
from tensororder_gb300.program import Program

NAMES = golden_names()


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_float64(name):
    doc = load_golden(name)
    prog = Program.from_dict(doc["program"])
    got = float(oracle.contract_sliced(prog))
    assert rel(got, doc["reference"]["float64"]) <= 1e-13


@pytest.mark.parametrize("name", [n for n in NAMES if "bigint" in load_golden(n)["reference"]])
def test_oracle_exact_count_matches_reference_bigint(name):
    doc = load_golden(name)
    prog = Program.from_dict(doc["program"])
    got = oracle.contract_sliced(prog, dtype=object)
    assert int(got) == int(doc["reference"]["bigint"])


@pytest.mark.parametrize("name", [n for n in NAMES if "brute_force" in load_golden(n)])
def test_reference_agrees_with_brute_force(name):
    doc = load_golden(name)
    assert rel(doc["reference"]["float64"], doc["brute_force"]) <= 1e-12


@pytest.mark.parametrize("name", [n for n in NAMES if "prefix_float64" in load_golden(n)["reference"]])
def test_oracle_slice_prefixes(name):
    doc = load_golden(name)
    prog = Program.from_dict(doc["program"])
    for k, want in enumerate(doc["reference"]["prefix_float64"], start=1):
        got = float(oracle.contract_sliced(prog, num_slice_limit=k))
        assert abs(got - want) <= 1e-13 * abs(doc["reference"]["float64"])


@pytest.mark.parametrize("name", NAMES)
def test_program_round_trip(name, tmp_path):
    doc = load_golden(name)
    prog = Program.from_dict(doc["program"])
    for suffix in (".json", ".json.gz"):
        p = tmp_path / ("p" + suffix)
        prog.dump(str(p))
        back = Program.load(str(p))
        assert back.to_dict() == prog.to_dict()
        for a, b in zip(prog.leaves, back.leaves):
            assert np.array_equal(a.parent(), b.parent())


def test_join_shapes_and_flops():
    prog = Program.from_dict(load_golden("vc50_bundled")["program"])
    shapes = oracle.join_shapes(prog)
    assert len(shapes) == prog.num_joins
    assert oracle.algorithmic_flops(prog) == sum(2 * m * n * k for m, n, k in shapes)


def test_validate_rejects_bad_programs():
    prog = Program.from_dict(load_golden("wvc18_s2")["program"])
    d = prog.to_dict()
    d2 = dict(d, postorder=d["postorder"][:-1])
    with pytest.raises(ValueError):
        Program.from_dict(d2)
    d3 = dict(d, slice_groups=[d["slice_groups"][0], d["slice_groups"][0]])
    with pytest.raises(ValueError):
        Program.from_dict(d3)
