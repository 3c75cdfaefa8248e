"""Exact integer counts from the int forms (the reference's ``bigint`` entry type).

The reference's ``bigint`` entry type contracts numpy object arrays of Python
integers (``numpy_apis.py:15-22``), so an unweighted count comes out exact
however large it is.  On the device the same integer is recovered from its
residues:

* the int form (``MODE_INT64``) gives the count modulo 2^64;
* the residue form (``MODE_MOD``) gives it modulo primes just below 2^28
  (small enough that its tiled kernel reduces once per 16 products);
* the split form's floating-point count bounds it: leaf values are
  non-negative in every form, so the count is a sum of non-negative terms,
  accurate to about 1e-6.  Enough primes are taken that 2^64 times their
  product exceeds twice that bound.  The residues are then combined by the
  Chinese remainder theorem into the unique integer of that symmetric range.

Leaves that are not all integers make the reference's object arithmetic
floating point (Python floats times ints), so the caller then returns the
plain FP64 count instead.
"""
from __future__ import annotations

import math

import numpy as np

WORD = 1 << 64


def _is_prime(n: int) -> bool:
    """Deterministic Miller-Rabin for n < 3,215,031,751 (bases 2, 3, 5, 7)."""
    if n < 2:
        return False
    for q in (2, 3, 5, 7):
        if n % q == 0:
            return n == q
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in (2, 3, 5, 7):
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def primes_below(limit: int, count: int):
    """The ``count`` largest primes below ``limit`` (descending)."""
    out, n = [], limit - 1
    while len(out) < count and n > 2:
        if _is_prime(n):
            out.append(n)
        n -= 1
    return out


# 64 primes below 2^28: 2^64 times their product exceeds 2^1850, beyond any
# bound an FP64 count can give.
MODULI = primes_below(1 << 28, 64)


def moduli_for(bound: float):
    """The primes needed so that 2^64 times their product exceeds 2 * bound + 1."""
    if not math.isfinite(bound):
        raise OverflowError("the count's magnitude exceeds the FP64 range; no residue set can be sized for it")
    need = 2 * int(math.ceil(bound)) + 2
    out, M = [], WORD
    for p in MODULI:
        if M > need:
            break
        out.append(p)
        M *= p
    if M <= need:
        raise OverflowError("the count needs more than %d residues" % len(MODULI))
    return out


def combine(word: int, residues, moduli) -> int:
    """The integer x with x = word (mod 2^64) and x = residues[i] (mod moduli[i]),
    taken in the symmetric range (-M/2, M/2] of M = 2^64 * prod(moduli)."""
    x, M = int(word) % WORD, WORD
    for r, p in zip(residues, moduli):
        # x + M * t = r (mod p)
        t = (int(r) - x) * pow(M % p, -1, p) % p
        x += M * t
        M *= p
    return x - M if x > M // 2 else x


def integer_leaves(program) -> bool:
    """True when every leaf value is an integer of magnitude below 2^63, so
    the integer forms compute the reference's exact ``bigint`` arithmetic."""
    for leaf in program.leaves:
        v = np.asarray(leaf.parent(), dtype=np.float64)
        if not np.all(np.isfinite(v)) or np.any(np.abs(v) >= 2.0 ** 63) or np.any(v != np.trunc(v)):
            return False
    return True


