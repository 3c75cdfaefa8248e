"""Pairwise contractions at the sweep's largest shapes, both forms.

The pairwise-contraction sweep covers ranks a, b up to 28 sharing k up to 14
indices (a + b - 2k <= 30, the reference's default rank limit).  Its largest
cases are too large for a full host contraction, so a seeded sample of 4096
output entries is recomputed on the host, each as an explicit K-long FP64 dot
product of the operands' fibres -- the value ``np.tensordot``
(``numpy_apis.py:42-43``) gives for that entry.  Tolerances are per entry:
1e-12 for the plain FP64 form, 1e-6 for the split form; every entry is
positive, so the relative error is well defined.  The long-K cases (K up to
2^14) are the ones where the split form's windowed accumulation matters.
"""
import numpy as np
import pytest

from tensororder_gb300 import run_sweep, runtime

pytestmark = pytest.mark.gpu

SHAPES = [(24, 22, 12), (26, 24, 12), (26, 25, 14), (28, 28, 14), (28, 16, 14), (22, 22, 9)]


@pytest.mark.parametrize("a,b,k", SHAPES)
@pytest.mark.parametrize("mode,tol", [(runtime.MODE_F64, 1e-12), (runtime.MODE_SPLIT, 1e-6)])
def test_large_pairwise_contraction(a, b, k, mode, tol, cuda):
    assert a + b - 2 * k <= 30
    prog = run_sweep.case(1000 + 37 * a + b + k, a, b, k)
    res, _, _ = run_sweep.run_case(prog, mode, repeats=1)
    assert run_sweep.sampled_check(prog, res, samples=4096, seed=a + b + k) <= tol
