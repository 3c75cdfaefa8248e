"""Pairwise contraction kernel against np.tensordot (the reference's
NumpyAPI.tensordot, numpy_apis.py:42-43): seeded random FP64 tensors with every
dimension 2, entries uniform in [0.5, 1.5], random ranks, shared-axis counts and
axis permutations.  Tolerance 1e-12 relative (max-norm)."""
import numpy as np
import pytest

from tensororder_gb300 import runtime

pytestmark = pytest.mark.gpu


def case(rng, ra, rb, k):
    a = rng.uniform(0.5, 1.5, size=(2,) * ra)
    b = rng.uniform(0.5, 1.5, size=(2,) * rb)
    axes_a = list(rng.permutation(ra)[:k])
    axes_b = list(rng.permutation(rb)[:k])
    return a, b, (axes_a, axes_b)


def check(a, b, axes, cuda):
    import torch

    want = np.tensordot(a, b, axes)
    got = runtime.tensordot_f64(torch.as_tensor(a, device=cuda), torch.as_tensor(b, device=cuda), axes)
    got = got.cpu().numpy()
    assert got.shape == want.shape
    scale = max(np.abs(want).max(), 1e-300)
    assert np.abs(got - want).max() / scale <= 1e-12


@pytest.mark.parametrize("seed", range(40))
def test_small_random(seed, cuda):
    rng = np.random.default_rng(seed)
    ra, rb = int(rng.integers(0, 10)), int(rng.integers(0, 10))
    k = int(rng.integers(0, min(ra, rb) + 1))
    check(*case(rng, ra, rb, k), cuda)


@pytest.mark.parametrize("ra,rb,k", [(10, 10, 5), (16, 16, 8), (14, 12, 6), (20, 14, 10), (18, 18, 12),
                                     (12, 20, 4), (9, 22, 8), (24, 16, 12), (8, 8, 0), (20, 20, 10)])
def test_sweep_shapes(ra, rb, k, cuda):
    rng = np.random.default_rng(ra * 1000 + rb * 10 + k)
    check(*case(rng, ra, rb, k), cuda)


def test_full_contraction_and_scalars(cuda):
    rng = np.random.default_rng(7)
    a = rng.uniform(0.5, 1.5, size=(2,) * 6)
    check(a, a, (list(range(6)), list(range(6))), cuda)
    s = np.array(1.25)
    check(s, a, ([], []), cuda)
    check(a, s, ([], []), cuda)
    check(s, s, ([], []), cuda)
