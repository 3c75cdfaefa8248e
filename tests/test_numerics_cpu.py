"""CPU checks of the bit-level arithmetic the split-form kernels use.

* TF32 rounding on the IEEE bit pattern, ``(bits + 0x1000) & 0xFFFFE000``
  (``tf32_rn`` in the tensor-core kernels), against round-to-nearest, ties away
  from zero, to 11 significant bits computed in exact rational arithmetic.
* The hi/lo split built on it: ``hi + lo`` recovers an FP32 value to 2^-22
  relative, the accuracy 3xTF32 products rely on.
"""
from fractions import Fraction

import numpy as np


def tf32_bits(x):
    b = np.asarray(x, dtype=np.float32).view(np.uint32)
    return ((b + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)


def tf32_exact(x):
    """Nearest value with 11 significant bits, ties away from zero."""
    x = float(x)
    if x == 0.0:
        return 0.0
    m, e = np.frexp(x)  # x = m * 2^e, 0.5 <= |m| < 1
    q = Fraction(float(m)) * 2 ** 11
    r = int(abs(q) + Fraction(1, 2))  # half away from zero on the magnitude
    return float(np.ldexp(np.sign(m) * r, int(e) - 11))


def test_bit_rounding_matches_exact_rounding():
    rng = np.random.default_rng(0)
    xs = np.concatenate([
        rng.uniform(0, 2, 4000), -rng.uniform(0, 2, 1000), rng.uniform(1e-30, 1e-20, 500),
        rng.uniform(1e20, 1e30, 500),
        # exact ties and the values next to them
        np.array([1 + 2 ** -11, 1 + 3 * 2 ** -11, 2 - 2 ** -12, 1.5 + 2 ** -11 - 2 ** -23, 1.0, 0.0]),
    ]).astype(np.float32)
    got = tf32_bits(xs)
    want = np.array([tf32_exact(x) for x in xs], dtype=np.float32)
    assert np.array_equal(got, want)


def test_hi_lo_split_accuracy():
    rng = np.random.default_rng(1)
    v = rng.uniform(1, 2, 100000).astype(np.float32)
    hi = tf32_bits(v)
    lo = tf32_bits(v - hi)
    err = np.abs((hi.astype(np.float64) + lo) - v.astype(np.float64)) / v
    assert err.max() <= 2.0 ** -22
