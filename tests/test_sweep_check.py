"""The sampled-entry check used for pairwise contractions too large for a
full host contraction (no GPU needed): on small cases it must agree with the
full ``np.tensordot`` result of the same inputs (``numpy_apis.py:42-43``) and
see a perturbation of a single entry's size."""
import numpy as np
import pytest

from tensororder_gb300 import run_sweep


@pytest.mark.parametrize("a,b,k", [(10, 9, 4), (8, 12, 6), (12, 6, 0), (9, 9, 9)])
def test_sampled_check_matches_full_contraction(a, b, k):
    prog = run_sweep.case(11 * a + b + k, a, b, k)
    full = run_sweep.host_result(prog)
    assert run_sweep.sampled_check(prog, full, samples=512) <= 1e-14
    bad = np.array(full, copy=True)
    bad *= 1 + 3e-8
    assert run_sweep.sampled_check(prog, bad, samples=512) > 1e-8


def test_operand_matrices_are_the_operands():
    prog = run_sweep.case(3, 7, 6, 3)
    X2, Y2 = run_sweep.operand_matrices(prog)
    assert X2.shape == (1 << 4, 1 << 3) and Y2.shape == (1 << 3, 1 << 3)
    full = run_sweep.host_result(prog).reshape(X2.shape[0], Y2.shape[0])
    assert np.allclose(X2 @ Y2.T, full, rtol=1e-14, atol=0)
